"""Seeded synthetic scenes for parity tests and benchmarks.

All geometry is z-up, in metres, built from a numpy PCG64 generator seeded by
the caller, so every run of a given (scene, seed) is byte-identical.

* `basic`, `hugeoverlap`: the two self-contained scenes of the reference's own
  test driver (lighter_test.cpp:183-306), rebuilt from their parameters.
* `obj_scene`: the reference's OBJ-fixture scenes (mesh1, mesh2, rad1;
  lighter_test.cpp:308-544) when given the fixture directory.
* `cornell` (C1), `mid` (C2), `large` (C3), `batch` (C4): procedural scenes
  with the shapes and sizes of the benchmark workloads; lightmap UVs come from
  per-face planar charts packed on a grid (`pack_faces`).
"""
from __future__ import annotations

import math
import os

import numpy as np

from .abi import LTR_LT_DIRECT, LTR_LT_POINT, LTR_LT_SPOT
from .scene import Instance, Light, Mesh, Part, SceneDesc


# ----------------------------------------------------------------------------- geometry

def yaw_matrix(yaw: float, tx=0.0, ty=0.0, tz=0.0, scale=(1.0, 1.0, 1.0)) -> np.ndarray:
    """Row-vector transform (v' = v M, translation in row 3), scale then yaw about z."""
    c, s = math.cos(yaw), math.sin(yaw)
    m = np.zeros((4, 4), np.float32)
    m[0, :3] = (c * scale[0], s * scale[0], 0)
    m[1, :3] = (-s * scale[1], c * scale[1], 0)
    m[2, :3] = (0, 0, scale[2])
    m[3, :3] = (tx, ty, tz)
    m[3, 3] = 1
    return m


def box_faces(sx, sy, sz, yaw=0.0, cx=0.0, cy=0.0, z0=0.0):
    """Six outward quads of a box standing on z=z0, yawed about its centre."""
    hx, hy = sx / 2, sy / 2
    corners = np.array([[-hx, -hy, 0], [hx, -hy, 0], [hx, hy, 0], [-hx, hy, 0],
                        [-hx, -hy, sz], [hx, -hy, sz], [hx, hy, sz], [-hx, hy, sz]], np.float64)
    c, s = math.cos(yaw), math.sin(yaw)
    rot = np.array([[c, s, 0], [-s, c, 0], [0, 0, 1]])
    corners = corners @ rot + np.array([cx, cy, z0])
    quads = [(0, 3, 2, 1), (4, 5, 6, 7), (0, 1, 5, 4), (1, 2, 6, 5), (2, 3, 7, 6), (3, 0, 4, 7)]
    return [corners[list(q)] for q in quads]


def icosphere(subdiv: int):
    """Unit icosphere: 20 * 4**subdiv triangles, as an (T,3,3) array."""
    t = (1 + 5 ** 0.5) / 2
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    v = [np.array(p, np.float64) / np.linalg.norm(p) for p in v]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
         (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
         (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    tris = [np.array([v[a], v[b], v[c]]) for a, b, c in f]
    for _ in range(subdiv):
        nt = []
        for tr in tris:
            a, b, c = tr
            ab = (a + b) / np.linalg.norm(a + b)
            bc = (b + c) / np.linalg.norm(b + c)
            ca = (c + a) / np.linalg.norm(c + a)
            nt += [np.array([a, ab, ca]), np.array([b, bc, ab]), np.array([c, ca, bc]), np.array([ab, bc, ca])]
        tris = nt
    return np.array(tris)


def _face_normal(poly):
    n = np.cross(poly[1] - poly[0], poly[2] - poly[0])
    ln = np.linalg.norm(n)
    return n / ln if ln > 0 else np.array([0, 0, 1.0])


def pack_faces(faces, lm_size: int, pad_texels: float = 2.0):
    """Per-face planar charts on a square grid: face k gets cell (k % g, k // g);
    its polygon is projected onto its own plane and scaled uniformly to fit the
    cell minus `pad_texels` of margin. Returns one (k,2) UV array per face."""
    g = max(1, int(math.ceil(math.sqrt(len(faces)))))
    cell = 1.0 / g
    # the margin shrinks to a quarter of the cell when cells get small
    pad = min(pad_texels, 0.25 * cell * lm_size) / lm_size
    inner = cell - 2 * pad
    if inner <= 0:
        raise ValueError(f"{len(faces)} faces do not fit a {lm_size}^2 lightmap")
    out = []
    for k, poly in enumerate(faces):
        n = _face_normal(poly)
        a = poly[1] - poly[0]
        a = a / np.linalg.norm(a)
        b = np.cross(n, a)
        uv = np.stack([(poly - poly[0]) @ a, (poly - poly[0]) @ b], 1)
        uv -= uv.min(0)
        ext = max(uv.max(), 1e-9)
        uv = uv / ext * inner
        cx, cy = k % g, k // g
        uv += np.array([cx * cell + pad, cy * cell + pad])
        out.append(uv)
    return out


def pack_faces_fast(faces, lm_size: int, pad_texels: float = 2.0):
    """Vectorised pack_faces for faces of equal vertex count (same layout and
    charts, evaluated with array operations; used by the generators of the
    large and batch workloads)."""
    F = np.asarray(faces, np.float64)                   # (k, m, 3)
    k = len(F)
    g = max(1, int(math.ceil(math.sqrt(k))))
    cell = 1.0 / g
    pad = min(pad_texels, 0.25 * cell * lm_size) / lm_size
    inner = cell - 2 * pad
    if inner <= 0:
        raise ValueError(f"{k} faces do not fit a {lm_size}^2 lightmap")
    n = np.cross(F[:, 1] - F[:, 0], F[:, 2] - F[:, 0])
    ln = np.linalg.norm(n, axis=1, keepdims=True)
    n = np.where(ln > 0, n / np.where(ln > 0, ln, 1), np.array([0, 0, 1.0]))
    a = F[:, 1] - F[:, 0]
    a = a / np.linalg.norm(a, axis=1, keepdims=True)
    b = np.cross(n, a)
    d = F - F[:, :1]
    uv = np.stack([np.einsum("kmc,kc->km", d, a), np.einsum("kmc,kc->km", d, b)], -1)
    uv -= uv.min(1, keepdims=True)
    ext = np.maximum(uv.max((1, 2)), 1e-9)[:, None, None]
    uv = uv / ext * inner
    idx = np.arange(k)
    uv += np.stack([(idx % g) * cell + pad, (idx // g) * cell + pad], 1)[:, None, :]
    return uv, n


def faces_to_part_fast(faces, lm_size, face_id0=0, shadow=1, pad_texels=2.0):
    """faces_to_part for triangles and quads through pack_faces_fast; faces are
    grouped by vertex count, each group packed into its own half of the map
    when both kinds are present."""
    tris = [f for f in faces if len(f) == 3]
    quads = [f for f in faces if len(f) == 4]
    groups = [(g_, m) for g_, m in ((tris, 3), (quads, 4)) if g_]
    P, N, T1, T2, I = [], [], [], [], []
    base, fid = 0, face_id0
    for gi, (grp, m) in enumerate(groups):
        uv, n = pack_faces_fast(grp, lm_size, pad_texels)
        if len(groups) == 2:             # left or right half
            uv = uv * np.array([0.5, 1.0]) + np.array([0.5 * gi, 0.0])
        k = len(grp)
        P.append(np.asarray(grp, np.float64).reshape(-1, 3))
        N.append(np.repeat(n, m, 0))
        T1.append(np.stack([np.repeat(fid + np.arange(k) + 0.5, m), np.zeros(k * m)], 1))
        T2.append(uv.reshape(-1, 2))
        fan = np.array([[0, j, j + 1] for j in range(1, m - 1)]).ravel()
        I.append((base + np.arange(k)[:, None] * m + fan[None, :]).ravel())
        base += k * m
        fid += k
    return Part(np.concatenate(P).astype(np.float32), np.concatenate(N).astype(np.float32),
                np.concatenate(T1).astype(np.float32), np.concatenate(T2).astype(np.float32),
                np.concatenate(I).astype(np.uint32), shadow)


def faces_to_part(faces, lm_size, face_id0=0, shadow=1, pad_texels=2.0):
    """Flat-shaded part: each face has its own vertices, normal and chart; uv1.u
    carries the global face id (face_id0 + k) for table-driven albedo."""
    uvs = pack_faces(faces, lm_size, pad_texels)
    P, N, T1, T2, I = [], [], [], [], []
    base = 0
    for k, (poly, uv) in enumerate(zip(faces, uvs)):
        n = _face_normal(poly)
        m = len(poly)
        P.append(poly)
        N.append(np.repeat(n[None], m, 0))
        T1.append(np.repeat(np.array([[face_id0 + k + 0.5, 0.0]]), m, 0))
        T2.append(uv)
        for j in range(1, m - 1):
            I += [base, base + j, base + j + 1]
        base += m
    return Part(np.concatenate(P).astype(np.float32), np.concatenate(N).astype(np.float32),
                np.concatenate(T1).astype(np.float32), np.concatenate(T2).astype(np.float32),
                np.array(I, np.uint32), shadow)


# ----------------------------------------------------------------------------- reference test scenes

def _quad_part(shadow=1, copies=1):
    pos = np.array([-1, -1, 0, 1, -1, 0, 1, 1, 0, -1, 1, 0], np.float32).reshape(4, 3)
    nrm = np.tile(np.array([0, 0, 1], np.float32), (4, 1))
    uv = np.array([0.1, 0.1, 0.9, 0.1, 0.9, 0.9, 0.1, 0.9], np.float32).reshape(4, 2)
    idx = np.tile(np.array([0, 1, 2, 2, 3, 0], np.uint32), copies)
    return Part(pos, nrm, uv, uv, idx, shadow)


def basic() -> SceneDesc:
    """Quad mesh, three instances, one point light (lighter_test.cpp:183-257)."""
    c, s = math.cos(0.5) * 0.2, math.sin(0.5) * 0.2
    m2 = np.array([[c, s, 0, 0], [-s, c, 0, 0], [0, 0, 0.2, 0], [0, 0, 0.5, 1]], np.float32)
    m3 = np.array([[1.9, 0, 0, 0], [0, 1.9, 0, 0], [0, 0, 1.9, 0], [0, 0, -0.5, 1]], np.float32)
    return SceneDesc(
        "basic", [Mesh("mesh1", [_quad_part()])],
        [Instance(0), Instance(0, m2), Instance(0, m3)],
        [Light(LTR_LT_POINT, (-0.4, -0.4, 1), color=(0.9, 0.1, 0.05), range=4.0, power=1.0,
               light_radius=0.1, shadow_sample_count=9)])


def hugeoverlap() -> SceneDesc:
    """16 copies of the quad's triangles, ten identical instances (lighter_test.cpp:259-306)."""
    return SceneDesc(
        "hugeoverlap", [Mesh("mesh1", [_quad_part(copies=16)])], [Instance(0) for _ in range(10)],
        [Light(LTR_LT_POINT, (-0.4, -0.4, 1), color=(0.9, 0.1, 0.05), range=4.0, power=1.0,
               light_radius=0.1, shadow_sample_count=9)])


def load_obj(path):
    """The fixture format of lighter_test.cpp:48-107 (v/vt/vn/f with v/t/n
    triplets, vt.y flipped, vertices deduplicated on exact (P,N,T))."""
    plist, nlist, tlist = [], [], []
    pos, nrm, tex, idx = [], [], [], []
    lookup = {}
    with open(path) as fh:
        for line in fh:
            tok = line.split()
            if not tok:
                continue
            if tok[0] == "v":
                plist.append(tuple(np.float32(x) for x in tok[1:4]))
            elif tok[0] == "vt":
                u, v = np.float32(tok[1]), np.float32(tok[2])
                tlist.append((u, np.float32(np.float32(1) - v)))
            elif tok[0] == "vn":
                nlist.append(tuple(np.float32(x) for x in tok[1:4]))
            elif tok[0] == "f":
                for vert in tok[1:4]:
                    a, b, c = (int(x) - 1 for x in vert.split("/"))
                    key = (plist[a], nlist[c], tlist[b])
                    if key not in lookup:
                        lookup[key] = len(pos)
                        pos.append(plist[a])
                        nrm.append(nlist[c])
                        tex.append(tlist[b])
                    idx.append(lookup[key])
    t = np.array(tex, np.float32)
    return Part(np.array(pos, np.float32), np.array(nrm, np.float32), t, t, np.array(idx, np.uint32), 1)


def obj_scene(name: str, fixture_dir: str) -> SceneDesc:
    """mesh1 / mesh2 / rad1 of lighter_test.cpp:308-544, from the OBJ fixtures."""
    def f(n):
        return os.path.join(fixture_dir, n)
    if name == "mesh1":
        return SceneDesc(
            "mesh1", [Mesh("mesh1", [load_obj(f("test-mesh.data"))])], [Instance(0)],
            [Light(LTR_LT_POINT, (-2.18, -4.04, 1.40), color=(0.9, 0.7, 0.5), range=16, power=1, light_radius=0.1,
                   shadow_sample_count=5),
             Light(LTR_LT_POINT, (2.18, 4.04, 1.40), color=(0.5, 0.7, 0.9), range=16, power=1, light_radius=0.1,
                   shadow_sample_count=5),
             Light(LTR_LT_SPOT, (0, 0, 1.60), (0, 0, -1), (1, 0, 0), (0.7, 0.1, 0.05), 16, 1, 0.1, 5, 45, 25, 0.5)],
            config={"ao_distance": 2.0})
    if name == "mesh2":
        return SceneDesc(
            "mesh2", [Mesh("mesh1", [load_obj(f("test-set2-mesh1.data"))]),
                      Mesh("mesh2", [load_obj(f("test-set2-mesh2.data"))])],
            [Instance(0), Instance(1, importance=0.3)],
            [Light(LTR_LT_POINT, (-2.18, -4.04, 1.40), color=(0.9, 0.7, 0.5), range=16, power=1, light_radius=0.2,
                   shadow_sample_count=5),
             Light(LTR_LT_POINT, (2.18, 4.04, 1.40), color=(0.5, 0.7, 0.9), range=16, power=1, light_radius=0.2,
                   shadow_sample_count=5),
             Light(LTR_LT_SPOT, (0, 0, 1.60), (0, 0, -1), (1, 0, 0), (0.7, 0.1, 0.05), 16, 1, 0.2, 5, 45, 25, 0.5),
             Light(LTR_LT_DIRECT, (0, 0, 0), (1, 1, 1), (0, 0, 0), (0.6, 0.55, 0.5), 1000, 1, 0.2, 1)],
            config={"ao_distance": 2.0, "global_size_factor": 4.0, "blur_size": 0.0, "generate_normalmap_data": 1})
    if name == "rad1":
        def red_wall(req):
            if req.position[0] <= -3 and req.normal[0] > 0.1:
                req.out_diffuse_color[0] = 0.5
                req.out_diffuse_color[1] = 0.05
                req.out_diffuse_color[2] = 0.02
            return True
        return SceneDesc(
            "rad1", [Mesh("mesh1", [load_obj(f("test-set2-mesh1.data"))])], [Instance(0, importance=0.4)],
            [Light(LTR_LT_POINT, (10.18, 0, 1.40), color=(0.99, 0.97, 0.95), range=24, power=1, light_radius=0.1,
                   shadow_sample_count=5)],
            config={"ao_distance": 2.0, "bounce_count": 2}, sample_fn_py=red_wall)
    raise KeyError(name)


# ----------------------------------------------------------------------------- benchmark scenes

def cornell(seed: int = 1, lm: int = 128, bounces: int = 1, ao: bool = False) -> SceneDesc:
    """C1: 10 m room of 6 walls (2 tris each, one mesh+instance per wall) and two
    boxes yawed by U(0,45 deg) (12 tris each): 36 triangles, 8 lightmaps of lm^2.
    Per-face albedo U(0.3,0.8) via the table sample_fn; 1 point light (RGB 1,
    radius 0.2, 16 samples) and 1 directional light (32 samples) through the
    open (non-shadowing) ceiling; `bounces` radiosity bounces, no AO."""
    rng = np.random.default_rng(seed)
    S = 10.0
    p = np.array
    walls = [
        ("floor", p([[0, 0, 0], [S, 0, 0], [S, S, 0], [0, S, 0]], float)),
        ("ceiling", p([[0, 0, S], [0, S, S], [S, S, S], [S, 0, S]], float)),
        ("wall_x0", p([[0, 0, 0], [0, S, 0], [0, S, S], [0, 0, S]], float)),
        ("wall_x1", p([[S, 0, 0], [S, 0, S], [S, S, S], [S, S, 0]], float)),
        ("wall_y0", p([[0, 0, 0], [0, 0, S], [S, 0, S], [S, 0, 0]], float)),
        ("wall_y1", p([[0, S, 0], [S, S, 0], [S, S, S], [0, S, S]], float)),
    ]
    meshes, insts = [], []
    fid = 0
    for name, quad in walls:
        part = faces_to_part([quad], lm, fid, shadow=0 if name == "ceiling" else 1)
        fid += 1
        meshes.append(Mesh(name, [part]))
        insts.append(Instance(len(meshes) - 1, ident=name))
    for k, (sx, sy, sz, cx, cy) in enumerate([(2.5, 2.5, 2.5, 3.2, 3.0), (2.5, 2.5, 5.0, 6.6, 6.4)]):
        yaw = math.radians(rng.uniform(0, 45))
        faces = box_faces(sx, sy, sz, yaw, cx, cy, 0.0)
        meshes.append(Mesh(f"box{k}", [faces_to_part(faces, lm, fid)]))
        fid += 6
        insts.append(Instance(len(meshes) - 1, ident=f"box{k}"))
    albedo = rng.uniform(0.3, 0.8, (fid, 3)).astype(np.float32)
    lights = [
        Light(LTR_LT_POINT, (5.0, 5.0, 8.5), color=(1, 1, 1), range=20.0, power=1.0, light_radius=0.2,
              shadow_sample_count=16),
        Light(LTR_LT_DIRECT, direction=(0.35, 0.25, 1.0), color=(0.8, 0.76, 0.7), range=40.0, power=1.0,
              light_radius=0.2, shadow_sample_count=32),
    ]
    cfg = {"bounce_count": bounces, "ao_distance": 2.0 if ao else 0.0}
    return SceneDesc(f"cornell{lm}", meshes, insts, lights, cfg, fixed_lm_size=(lm, lm),
                     sample_table=(albedo, None), seed=seed)


def mid(seed: int = 1, lm: int = 1024, n_boxes: int = 400, n_spheres: int = 50, bounces: int = 2,
        ao_rays: int = 32) -> SceneDesc:
    """C2: 200x200 m ground, `n_boxes` boxes (sizes U(0.5,8) m, yaw U(0,360 deg))
    and `n_spheres` 320-tri icospheres; 4 instances with lm^2 lightmaps (ground,
    two box groups, spheres); 8 point + 2 spot lights (cone U(20,60 deg)), 64
    shadow samples each; AO `ao_rays` rays of radius 2 m; `bounces` bounces."""
    rng = np.random.default_rng(seed)
    H = 100.0
    ground = [np.array([[-H, -H, 0], [H, -H, 0], [H, H, 0], [-H, H, 0]], float)]
    box_groups = [[], []]
    for k in range(n_boxes):
        sx, sy, sz = rng.uniform(0.5, 8.0, 3)
        cx, cy = rng.uniform(-H + 5, H - 5, 2)
        yaw = rng.uniform(0, 2 * math.pi)
        box_groups[k * 2 // max(n_boxes, 1)] += box_faces(sx, sy, sz, yaw, cx, cy, 0.0)
    unit = icosphere(2)
    spheres = []
    for _ in range(n_spheres):
        r = rng.uniform(1.0, 4.0)
        c = np.array([*rng.uniform(-H + 5, H - 5, 2), r])
        spheres += [tri * r + c for tri in unit]
    groups = [("ground", ground), ("boxes_a", box_groups[0]), ("boxes_b", box_groups[1]), ("spheres", spheres)]
    meshes, insts, fid = [], [], 0
    for name, faces in groups:
        if not faces:
            continue
        meshes.append(Mesh(name, [faces_to_part(faces, lm, fid, pad_texels=1.5)]))
        fid += len(faces)
        insts.append(Instance(len(meshes) - 1, ident=name))
    albedo = rng.uniform(0.3, 0.8, (fid, 3)).astype(np.float32)
    lights = []
    for _ in range(8):
        lights.append(Light(LTR_LT_POINT, (*rng.uniform(-90, 90, 2), rng.uniform(4, 12)),
                            color=tuple(rng.uniform(0.5, 1.0, 3)), range=float(rng.uniform(30, 60)), power=1.0,
                            light_radius=0.2, shadow_sample_count=64))
    for _ in range(2):
        out = rng.uniform(20, 60)
        d = np.array([rng.uniform(-0.3, 0.3), rng.uniform(-0.3, 0.3), -1.0])
        lights.append(Light(LTR_LT_SPOT, (*rng.uniform(-80, 80, 2), rng.uniform(8, 15)), tuple(d / np.linalg.norm(d)),
                            (1, 0, 0), tuple(rng.uniform(0.5, 1.0, 3)), float(rng.uniform(40, 60)), 1.0, 0.2, 64,
                            float(out), float(out * 0.6), 1.0))
    cfg = {"bounce_count": bounces, "ao_distance": 2.0 if ao_rays else 0.0, "ao_num_samples": max(ao_rays, 1)}
    return SceneDesc(f"mid{lm}", meshes, insts, lights, cfg, fixed_lm_size=(lm, lm),
                     sample_table=(albedo, None), seed=seed)


def _value_noise(x, y, rng_table):
    """Smooth value noise on the integer lattice (hashed through a 256-entry
    permutation of seeded random values), bilinear with a quintic fade."""
    perm, vals = rng_table
    xi, yi = np.floor(x).astype(np.int64), np.floor(y).astype(np.int64)
    fx, fy = x - xi, y - yi
    fx = fx * fx * fx * (fx * (fx * 6 - 15) + 10)
    fy = fy * fy * fy * (fy * (fy * 6 - 15) + 10)

    def h(ix, iy):
        return vals[perm[(perm[ix & 255] + iy) & 255]]

    a, b = h(xi, yi), h(xi + 1, yi)
    c, d = h(xi, yi + 1), h(xi + 1, yi + 1)
    return (a * (1 - fx) + b * fx) * (1 - fy) + (c * (1 - fx) + d * fx) * fy


def fbm_heights(rng, nx, ny, spacing, octaves=6, base_period=256.0, amplitude=60.0):
    """(ny+1, nx+1) heights of a seeded fBm: octave k has period base/2^k and weight 0.5^k."""
    table = (rng.permutation(256), rng.uniform(-1.0, 1.0, 256))
    xs = np.arange(nx + 1) * spacing
    ys = np.arange(ny + 1) * spacing
    X, Y = np.meshgrid(xs, ys)
    z = np.zeros_like(X)
    for k in range(octaves):
        f = (2.0 ** k) / base_period
        z += (0.5 ** k) * _value_noise(X * f + 17.3 * k, Y * f - 9.1 * k, table)
    return z * amplitude


def large(seed: int = 1, lm: int = 2048, grid=(1024, 512), tiles=(4, 4), n_rocks: int = 2000, n_points: int = 32,
          ao_rays: int = 64, bounces: int = 3, spacing: float = 2.0) -> SceneDesc:
    """C3: seeded fBm heightfield terrain (6 octaves, grid[0] x grid[1] quads =
    2 * grid[0] * grid[1] triangles; 1024 x 512 -> 1.05M) cut into tiles[0] x
    tiles[1] instances, each with an lm^2 lightmap, plus `n_rocks` 80-triangle
    icospheres (scale lognormal(0, 0.5)) scattered on it; every rock is packed
    into a strip of its tile's lightmap. 1 directional light (128 samples) and
    `n_points` point lights; AO `ao_rays` rays of radius 2 m; `bounces`
    radiosity bounces."""
    rng = np.random.default_rng(seed)
    nx, ny = grid
    tx, ty = tiles
    Z = fbm_heights(rng, nx, ny, spacing)
    W, D = nx * spacing, ny * spacing

    def height_at(x, y):
        i = np.clip((x / spacing).astype(int), 0, nx - 1)
        j = np.clip((y / spacing).astype(int), 0, ny - 1)
        return Z[j, i]

    # rocks: positions, scales, unit icosphere (80 triangles)
    unit = icosphere(1)
    unit_n = np.stack([_face_normal(f) for f in unit])
    chart_cache = {}
    rx, ry = rng.uniform(0, W, n_rocks), rng.uniform(0, D, n_rocks)
    rs = np.exp(rng.normal(0.0, 0.5, n_rocks))
    rz = height_at(rx, ry) + 0.3 * rs
    qx, qy = nx // tx, ny // ty
    strip = 0.125                  # lightmap fraction (v) that holds the tile's rocks
    margin = 2.0 / lm
    meshes, insts = [], []
    n_faces = 0
    for t_y in range(ty):
        for t_x in range(tx):
            i0, j0 = t_x * qx, t_y * qy
            ii, jj = np.meshgrid(np.arange(qx + 1), np.arange(qy + 1))
            gx, gy = (i0 + ii) * spacing, (j0 + jj) * spacing
            gz = Z[j0:j0 + qy + 1, i0:i0 + qx + 1]
            P = np.stack([gx, gy, gz], -1).reshape(-1, 3)
            # vertex normals from central differences of the heightfield
            zc = Z[max(j0 - 1, 0):j0 + qy + 2, max(i0 - 1, 0):i0 + qx + 2]
            dzdx = np.gradient(zc, spacing, axis=1)[(1 if j0 > 0 else 0):, (1 if i0 > 0 else 0):][:qy + 1, :qx + 1]
            dzdy = np.gradient(zc, spacing, axis=0)[(1 if j0 > 0 else 0):, (1 if i0 > 0 else 0):][:qy + 1, :qx + 1]
            N = np.stack([-dzdx, -dzdy, np.ones_like(dzdx)], -1).reshape(-1, 3)
            N /= np.linalg.norm(N, axis=1, keepdims=True)
            u = margin + ii / qx * (1 - 2 * margin)
            v = margin + jj / qy * (1 - strip - 2 * margin)
            T2 = np.stack([u, v], -1).reshape(-1, 2)
            T1 = np.tile(np.array([[n_faces + 0.5, 0.0]]), (len(P), 1))
            n_faces += 1
            a = (jj[:-1, :-1] * (qx + 1) + ii[:-1, :-1]).ravel()
            b, c, d = a + 1, a + qx + 2, a + qx + 1
            I = np.stack([a, b, c, a, c, d], 1).ravel()
            parts = [Part(P.astype(np.float32), N.astype(np.float32), T1.astype(np.float32), T2.astype(np.float32),
                          I.astype(np.uint32), 1)]
            # this tile's rocks, each a cell of the strip with per-face charts
            sel = np.nonzero((rx >= i0 * spacing) & (rx < (i0 + qx) * spacing) &
                             (ry >= j0 * spacing) & (ry < (j0 + qy) * spacing))[0]
            if len(sel):
                cols = max(1, int(math.ceil(math.sqrt(len(sel) / strip))))
                rows = int(math.ceil(len(sel) / cols))
                cw, ch = 1.0 / cols, strip / rows
                cell_px = int(min(cw, ch) * lm)
                # a rock is a scaled, translated unit icosphere: its charts and face normals are
                # the unit sphere's, computed once per cell size
                key = max(cell_px, 8)
                if key not in chart_cache:
                    chart_cache[key] = np.stack(pack_faces(list(unit), key, pad_texels=1.0))   # (80, 3, 2)
                uv_unit = chart_cache[key]
                k = np.arange(len(sel))
                corner = np.stack([(k % cols) * cw, 1 - strip + (k // cols) * ch], 1)          # (m, 2)
                sc = min(cw, ch)
                RP = unit[None] * rs[sel][:, None, None, None] + np.stack([rx[sel], ry[sel], rz[sel]], 1)[:, None, None]
                R2 = uv_unit[None] * sc + corner[:, None, None]
                RN = np.broadcast_to(unit_n[None, :, None, :], RP.shape)
                R1 = np.zeros(RP.shape[:3] + (2,))
                R1[..., 0] = (n_faces + k + 0.5)[:, None, None]
                n_faces += len(sel)
                parts.append(Part(RP.reshape(-1, 3).astype(np.float32), RN.reshape(-1, 3).astype(np.float32),
                                  R1.reshape(-1, 2).astype(np.float32), R2.reshape(-1, 2).astype(np.float32),
                                  np.arange(RP.shape[0] * RP.shape[1] * 3, dtype=np.uint32), 1))
            meshes.append(Mesh(f"tile{t_x}_{t_y}", parts))
            insts.append(Instance(len(meshes) - 1, ident=f"tile{t_x}_{t_y}"))
    albedo = rng.uniform(0.3, 0.8, (n_faces, 3)).astype(np.float32)
    lights = [Light(LTR_LT_DIRECT, direction=(0.3, 0.2, 1.0), color=(1.0, 0.95, 0.85), range=400.0, power=1.0,
                    light_radius=0.5, shadow_sample_count=128)]
    for _ in range(n_points):
        x, y = rng.uniform(0, W), rng.uniform(0, D)
        lights.append(Light(LTR_LT_POINT, (x, y, float(height_at(np.array([x]), np.array([y]))[0]) + rng.uniform(5, 20)),
                            color=tuple(rng.uniform(0.5, 1.0, 3)), range=float(rng.uniform(60, 120)), power=1.0,
                            light_radius=0.3, shadow_sample_count=16))
    cfg = {"bounce_count": bounces, "ao_distance": 2.0 if ao_rays else 0.0, "ao_num_samples": max(ao_rays, 1)}
    return SceneDesc(f"large{lm}", meshes, insts, lights, cfg, fixed_lm_size=(lm, lm),
                     sample_table=(albedo, None), seed=seed)


def batch_scene(seed: int) -> SceneDesc:
    """One scene of the C4 batch: a ground quad with boxes and 80-triangle
    icospheres up to a triangle count drawn lognormal (median 2k, clipped to
    200..20k); one instance per object group; a square lightmap whose side is
    log-uniform in [64, 512]; 1-8 point lights with 16-64 samples; AO 16 rays;
    no radiosity."""
    rng = np.random.default_rng(seed)
    target = int(np.clip(np.exp(rng.normal(math.log(2000.0), 0.8)), 200, 20000))
    lm = int(round(math.exp(rng.uniform(math.log(64), math.log(512)))))
    H = 30.0
    ground = [np.array([[-H, -H, 0], [H, -H, 0], [H, H, 0], [-H, H, 0]], float)]
    boxes, spheres = [], []
    unit = icosphere(1)
    n_tris = 2
    while n_tris < target:
        if rng.uniform() < 0.5:
            sx, sy, sz = rng.uniform(0.5, 5.0, 3)
            cx, cy = rng.uniform(-H + 3, H - 3, 2)
            boxes += box_faces(sx, sy, sz, rng.uniform(0, 2 * math.pi), cx, cy, 0.0)
            n_tris += 12
        else:
            r = rng.uniform(0.5, 2.5)
            c = np.array([*rng.uniform(-H + 3, H - 3, 2), r])
            spheres += [tri * r + c for tri in unit]
            n_tris += 80
    groups = [("ground", ground), ("boxes", boxes), ("spheres", spheres)]
    meshes, insts, fid = [], [], 0
    for name, faces in groups:
        if not faces:
            continue
        meshes.append(Mesh(name, [faces_to_part_fast(faces, lm, fid, pad_texels=1.0)]))
        fid += len(faces)
        insts.append(Instance(len(meshes) - 1, ident=name))
    albedo = rng.uniform(0.3, 0.8, (fid, 3)).astype(np.float32)
    lights = []
    for _ in range(int(rng.integers(1, 9))):
        lights.append(Light(LTR_LT_POINT, (*rng.uniform(-H, H, 2), rng.uniform(3, 10)),
                            color=tuple(rng.uniform(0.5, 1.0, 3)), range=float(rng.uniform(15, 40)), power=1.0,
                            light_radius=0.2, shadow_sample_count=int(rng.integers(16, 65))))
    cfg = {"bounce_count": 0, "ao_distance": 2.0, "ao_num_samples": 16}
    return SceneDesc(f"batch{seed}", meshes, insts, lights, cfg, fixed_lm_size=(lm, lm),
                     sample_table=(albedo, None), seed=seed)
