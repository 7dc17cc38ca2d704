"""The CPU oracle port against the reference's own outputs.

The golden fixtures (tests/golden/*.npz, made by make_golden.py from the
unmodified reference build) pin the oracle: it must reproduce them bit for
bit. Where the reference sources are present, the oracle is also compared
with a live reference build on the reference's own test scenes
(lighter_test.cpp:183-544) and with its OBJ fixtures.
"""
import os

import numpy as np
import pytest

from conftest import REF_SRC, ROOT

from lighter_gb300 import scenes
from lighter_gb300.scene import bake

GOLDEN = os.path.join(ROOT, "tests", "golden")


def _cases():
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


MG = _cases()


@pytest.mark.parametrize("name", list(MG.CASES))
def test_oracle_matches_golden(oracle, name):
    factory, samples = MG.CASES[name]
    res = bake(oracle, factory(), threads=1)
    got = MG.result_arrays(res, samples)
    want = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    assert sorted(got) == sorted(want.files)
    for k in want.files:
        np.testing.assert_array_equal(got[k], want[k], err_msg=f"{name}:{k}")


def test_oracle_threads_deterministic(oracle):
    """Multi-threaded oracle runs give the single-threaded result (AO random
    offsets are drawn in the single-threaded order)."""
    d = scenes.cornell(4, lm=32, bounces=0, ao=True)
    a = bake(oracle, d, threads=1)
    b = bake(oracle, d, threads=4)
    for x, y in zip(a.lightmaps, b.lightmaps):
        np.testing.assert_array_equal(x[3], y[3])


def _compare_libs(a, b, desc):
    ra = bake(a, desc, threads=1)
    rb = bake(b, desc, threads=1)
    assert len(ra.lightmaps) == len(rb.lightmaps)
    for x, y in zip(ra.lightmaps, rb.lightmaps):
        np.testing.assert_array_equal(x[3], y[3])
        if x[4] is not None:
            np.testing.assert_array_equal(x[4], y[4])
    for x, y in zip(ra.debug, rb.debug):
        for k in x:
            np.testing.assert_array_equal(x[k], y[k])
    np.testing.assert_array_equal(ra.sample_colors, rb.sample_colors)


@pytest.mark.parametrize("name", ["basic", "hugeoverlap"])
def test_oracle_vs_reference_builtin_scenes(oracle, ref, name):
    _compare_libs(ref, oracle, getattr(scenes, name)())


@pytest.mark.parametrize("name", ["mesh1", "rad1"])
def test_oracle_vs_reference_obj_fixtures(oracle, ref, name):
    fixtures = os.path.join(REF_SRC, "bin")
    if not os.path.isdir(fixtures):
        pytest.skip("reference fixtures not present")
    _compare_libs(ref, oracle, scenes.obj_scene(name, fixtures))


def test_reference_links_only_occluded_pairs(ref, oracle):
    """The reference keeps a radiosity link only when VisibilityTest() finds
    an occluder (lighter.cpp:751); the oracle restates that predicate."""
    from lighter_gb300.scene import Instance, Light, Mesh, SceneDesc
    q = scenes.faces_to_part([np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]], float)], 8)
    q2 = scenes.faces_to_part([np.array([[0, 0, 2], [0, 1, 2], [1, 1, 2], [1, 0, 2]], float)], 8)
    blk = scenes.faces_to_part([np.array([[-1, -1, 1], [2, -1, 1], [2, 2, 1], [-1, 2, 1]], float)], 8)
    counts = {}
    for lib_name, lib in (("ref", ref), ("orc", oracle)):
        for occl in (False, True):
            meshes = [Mesh("a", [q]), Mesh("b", [q2])] + ([Mesh("c", [blk])] if occl else [])
            insts = [Instance(i) for i in range(len(meshes))]
            d = SceneDesc("links", meshes, insts, [Light(1, (0.5, 0.5, 1.0), range=5.0)], {"bounce_count": 1},
                          fixed_lm_size=(8, 8))
            seen = {}

            class Spy:
                def __getattr__(self, n):
                    if n == "ltr_DestroyScene":
                        return lambda s: (seen.__setitem__("n", lib.ltrdbg_RadLinkCount(s)), lib.ltr_DestroyScene(s))
                    return getattr(lib, n)
            bake(Spy(), d)
            counts[(lib_name, occl)] = seen["n"]
    assert counts[("ref", False)] == 0 and counts[("ref", True)] > 0
    assert counts[("orc", False)] == counts[("ref", False)]
    assert counts[("orc", True)] == counts[("ref", True)]
