"""LTRG_ISECT_WATERTIGHT: the watertight segment/triangle test (Woop, Benthin
and Wald 2013) in place of the reference's IntersectLineSegmentTriangle
(lighter_math.cpp:315-354), for every ray query of the bake.

  - Leak test: segments from inside closed meshes out through their vertices
    and shared edges (the cases where the reference's inclusive barycentric
    test can miss both triangles of an edge) all hit in watertight mode.
  - Against the reference-semantics oracle: AO rays and sampled shadow rays
    flip hit/miss for fewer than 0.1% of the rays.
  - Against the oracle's restatement of the same mode: the same bars as the
    reference mode's parity tests.
"""
import os

import numpy as np
import pytest

from lighter_gb300 import ext, scenes
from lighter_gb300.scene import bake

pytestmark = pytest.mark.gpu

RAY_FLIP_FRAC = 1e-3


def _closed_meshes():
    """(triangles (n, 9), interior point) of a scaled, offset icosphere and of a cube."""
    sph = (scenes.icosphere(3) * 3.0 + np.array([10.25, -4.5, 2.125])).astype(np.float32)
    c = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]], np.float32)
    c = c * np.float32(2.5) + np.float32(-1.25)
    quads = [(0, 3, 2, 1), (4, 5, 6, 7), (0, 1, 5, 4), (1, 2, 6, 5), (2, 3, 7, 6), (3, 0, 4, 7)]
    cube = []
    for a, b, cc, d in quads:
        cube += [[c[a], c[b], c[cc]], [c[a], c[cc], c[d]]]
    return [(sph.reshape(-1, 9), np.array([10.25, -4.5, 2.125], np.float32) + np.float32(0.01)),
            (np.array(cube, np.float32).reshape(-1, 9), np.array([0.01, -0.02, 0.03], np.float32))]


def _targets(tri, center):
    """Points beyond every vertex and every edge midpoint, seen from `center`."""
    t = tri.reshape(-1, 3, 3).astype(np.float64)
    pts = [t.reshape(-1, 3)]
    for i, j in ((0, 1), (1, 2), (2, 0)):
        pts.append((t[:, i] + t[:, j]) * 0.5)
    p = np.unique(np.concatenate(pts), axis=0)
    return center + (p - center) * 2.0


def test_closed_meshes_do_not_leak(gpu):
    leaks = {}
    for tri, center in _closed_meshes():
        ends = _targets(tri, center.astype(np.float64)).astype(np.float32)
        seg = np.concatenate([np.broadcast_to(center, ends.shape), ends], axis=1)
        r_wt = ext.trace_segments(gpu, tri, seg, ext.LTRG_ISECT_WATERTIGHT)
        r_ref = ext.trace_segments(gpu, tri, seg, ext.LTRG_ISECT_REFERENCE)
        assert int((r_wt >= 1.0).sum()) == 0, f"{int((r_wt >= 1.0).sum())} of {len(seg)} segments leak"
        # the hit lies near the middle of each segment (the target is at twice the distance)
        assert float(np.abs(r_wt - 0.5).max()) < 0.01
        leaks[len(tri)] = int((r_ref >= 1.0).sum())
        both = (r_ref < 1.0)
        assert np.allclose(r_wt[both], r_ref[both], atol=1e-5)
    print("reference-test leaks (triangles: segments):", leaks)


def _ray_stats(rg, ro, ns):
    ao_tot = ao_flip = sh_tot = sh_flip = 0
    for a, b in zip(rg.debug, ro.debug):
        if "ao" in a and "ao" in b and a["ao"].size:
            ao_tot += a["ao"].size
            ao_flip += int(((a["ao"] < 1.0) != (b["ao"] < 1.0)).sum())
        if "vis" in a and a["vis"].size:
            both = (a["vis"] >= 0) & (b["vis"] >= 0)
            ha = np.rint((1.0 - a["vis"]) * ns).astype(np.int64)
            hb = np.rint((1.0 - b["vis"]) * ns).astype(np.int64)
            sh_tot += int((np.broadcast_to(ns, both.shape) * both).sum())
            sh_flip += int(np.abs(ha - hb)[both].sum())
    return ao_tot, ao_flip, sh_tot, sh_flip


@pytest.mark.parametrize("name", ["cornell32", "mid128"])
def test_watertight_rays_against_the_oracle(gpu, oracle, name):
    from test_gpu_parity import compare
    if name == "cornell32":
        d = scenes.cornell(4, lm=32, bounces=0, ao=True)
    else:
        d = scenes.mid(4, lm=128, n_boxes=24, n_spheres=3, bounces=0, ao_rays=8)
    ns = np.array([max(1, L.shadow_sample_count) for L in d.lights], np.int64)[:, None]
    wt = {"intersect_mode": 1, "shadow_mode": 1}
    rg = bake(gpu, d, gpu_options=wt)
    ro_ref = bake(oracle, d, threads=os.cpu_count() or 1, gpu_options={"shadow_mode": 1})
    ro_wt = bake(oracle, d, threads=os.cpu_count() or 1, gpu_options=wt)
    ao_tot, ao_flip, sh_tot, sh_flip = _ray_stats(rg, ro_ref, ns)
    assert ao_tot > 0 and sh_tot > 0
    assert ao_flip <= RAY_FLIP_FRAC * ao_tot, f"{ao_flip} of {ao_tot} AO rays flip against the reference test"
    assert sh_flip <= RAY_FLIP_FRAC * sh_tot, f"{sh_flip} of {sh_tot} shadow rays flip against the reference test"
    print(f"{name} watertight vs reference test: AO {ao_flip}/{ao_tot}, shadow rays {sh_flip}/{sh_tot}")
    ao_tot, ao_flip, sh_tot, sh_flip = _ray_stats(rg, ro_wt, ns)
    assert ao_flip <= RAY_FLIP_FRAC * ao_tot and sh_flip <= RAY_FLIP_FRAC * sh_tot
    print(f"{name} watertight vs the oracle's watertight: AO {ao_flip}/{ao_tot}, shadow rays {sh_flip}/{sh_tot}")
    compare(rg, ro_wt, f"watertight_{name}")
