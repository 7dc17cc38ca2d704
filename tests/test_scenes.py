"""The seeded scene generators against the workloads they stand for (CPU only).

cornell: 36 triangles (6 walls x 2, 2 boxes x 12), 8 lightmaps, 1 point + 1
directional light, albedo U(0.3, 0.8) per face. mid: 200 x 200 m ground, 400
boxes and 50 320-triangle icospheres (about 21k triangles), 8 point + 2 spot
lights, AO 32 rays of 2 m. large: 1024 x 512 terrain quads (1.05M triangles)
in 16 tiles plus 2000 80-triangle rocks (about 1.2M), 16 lightmaps of 2048^2, 1
directional + 32 point lights, AO 64 rays. batch: 256 scenes with 200..20k
triangles, lightmap sides in [64, 512], 1-8 point lights, AO 16 rays. The multi-RHS
room (C5): 32,768 patches of a furnished room (about 67k triangles), 64 emitter
subsets as 192 RGB right-hand sides.
Seeds give the same scene every time.
"""
import numpy as np

from lighter_gb300 import scenes

POINT, SPOT, DIRECTIONAL = 1, 2, 3


def _types(d):
    return [L.type for L in d.lights]


def test_cornell():
    d = scenes.cornell(1, lm=128)
    assert d.triangle_count() == 36
    assert len(d.instances) == 8 and d.fixed_lm_size == (128, 128)
    assert sorted(_types(d)) == [POINT, DIRECTIONAL]
    diffuse = d.sample_table[0]
    assert diffuse.min() >= 0.3 and diffuse.max() <= 0.8


def test_mid():
    d = scenes.mid(1, lm=1024)
    assert d.triangle_count() == 2 + 400 * 12 + 50 * 320
    assert len(d.instances) == 4 and d.fixed_lm_size == (1024, 1024)
    assert _types(d).count(POINT) == 8 and _types(d).count(SPOT) == 2
    for L in d.lights:
        if L.type == SPOT:
            assert 20.0 <= L.spot_angle_out <= 60.0
    assert d.config["ao_num_samples"] == 32 and d.config["ao_distance"] == 2.0
    assert d.config["bounce_count"] == 2


def test_large():
    d = scenes.large(1, lm=2048)
    assert d.triangle_count() == 2 * 1024 * 512 + 2000 * 80
    assert len(d.instances) == 16 and d.fixed_lm_size == (2048, 2048)
    assert _types(d).count(DIRECTIONAL) == 1 and _types(d).count(POINT) == 32
    assert d.config["ao_num_samples"] == 64 and d.config["bounce_count"] == 3


def test_batch_scenes():
    tris, sides = [], []
    for s in range(1, 257):
        d = scenes.batch_scene(s)
        tris.append(d.triangle_count())
        sides.append(d.fixed_lm_size[0])
        assert d.fixed_lm_size[0] == d.fixed_lm_size[1]
        assert 1 <= len(d.lights) <= 8 and set(_types(d)) == {POINT}
        assert d.config["ao_num_samples"] == 16 and d.config.get("bounce_count", 0) == 0
    tris, sides = np.array(tris), np.array(sides)
    assert tris.min() >= 200 and tris.max() <= 20000 + 400   # objects are whole: a group may pass the target
    assert 1000 <= np.median(tris) <= 4000                  # lognormal around 2k
    assert sides.min() >= 64 and sides.max() <= 512 and len(set(sides.tolist())) > 20


def test_generators_are_deterministic():
    a, b = scenes.mid(3, lm=64), scenes.mid(3, lm=64)
    for ia, ib in zip(a.instances, b.instances):
        np.testing.assert_array_equal(ia.matrix, ib.matrix)
    for ma, mb in zip(a.meshes, b.meshes):
        for pa, pb in zip(ma.parts, mb.parts):
            np.testing.assert_array_equal(pa.positions, pb.positions)
            np.testing.assert_array_equal(pa.indices, pb.indices)
    assert [L.position for L in a.lights] == [L.position for L in b.lights]


def test_multi_rhs_room():
    # the C5 patch set: a furnished room of about 60k triangles, 32,768 patches, 64 emitter
    # subsets as RGB right-hand sides (R = 192); unit normals, positive areas, albedo U(0.3, 0.8)
    from lighter_gb300 import patches
    sc = patches.room(seed=1, n_patches=32768, n_configs=64)
    n = len(sc["pos"])
    assert n == 32768 and sc["emission"].shape == (n, 192)
    assert 50_000 <= len(sc["tri"]) <= 80_000
    np.testing.assert_allclose(np.linalg.norm(sc["nrm"], axis=1), 1.0, rtol=1e-5)
    assert (sc["area"] > 0).all()
    assert sc["albedo"].min() >= 0.3 and sc["albedo"].max() <= 0.8
    lit = (sc["emission"] > 0).any(axis=0)
    assert lit.all()                                  # every configuration lights something
    b = patches.room(seed=1, n_patches=32768, n_configs=64)
    np.testing.assert_array_equal(sc["pos"], b["pos"])
    np.testing.assert_array_equal(sc["emission"], b["emission"])
