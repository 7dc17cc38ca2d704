"""Launch shapes of the trace kernels (ltrg_Tuning) and the autotuner."""
import ctypes as C

import numpy as np
import pytest

from lighter_gb300 import ext, scenes
from lighter_gb300.scene import bake, ingest


def _get(lib, dev=0):
    t = ext.Tuning()
    assert lib.ltrg_GetTuning(dev, C.byref(t))
    return t


def test_tuning_defaults_and_validation(gpu):
    lib = gpu
    saved = _get(lib)
    try:
        t = _get(lib)
        assert (t.direct_block, t.direct_blocks_per_sm, t.ao_block, t.ao_blocks_per_sm) != (0, 0, 0, 0)
        bad = ext.Tuning()
        C.memmove(C.byref(bad), C.byref(t), C.sizeof(t))
        bad.direct_block = 100                       # not a multiple of 32
        assert lib.ltrg_SetTuning(0, C.byref(bad)) == 0
        bad.direct_block = 1024                      # above 512
        assert lib.ltrg_SetTuning(0, C.byref(bad)) == 0
        bad.direct_block, bad.ao_blocks_per_sm = 64, 0
        assert lib.ltrg_SetTuning(0, C.byref(bad)) == 0
        bad.ao_blocks_per_sm, bad.ao_order = 8, 3   # no such order
        assert lib.ltrg_SetTuning(0, C.byref(bad)) == 0
        bad.ao_order, bad.direct_stack = 1, 5       # stacks: 0, 4, 8 or 16 shared-memory entries
        assert lib.ltrg_SetTuning(0, C.byref(bad)) == 0
        bad.direct_stack, bad.ao_chunk = 8, 9       # 1..8 rays per lane per fetch
        assert lib.ltrg_SetTuning(0, C.byref(bad)) == 0
        bad.ao_chunk, bad.direct_packet = 1, 2
        assert lib.ltrg_SetTuning(0, C.byref(bad)) == 0
        bad.direct_packet, bad.direct_regs = 1, 4  # register budgets 0..3
        assert lib.ltrg_SetTuning(0, C.byref(bad)) == 0
        assert lib.ltrg_SetTuning(-1, C.byref(t)) == 0
        ok = ext.Tuning()
        C.memmove(C.byref(ok), C.byref(t), C.sizeof(t))
        ok.direct_block, ok.direct_blocks_per_sm = 64, 4
        assert lib.ltrg_SetTuning(0, C.byref(ok)) == 1
        got = _get(lib)
        assert (got.direct_block, got.direct_blocks_per_sm) == (64, 4)
        assert lib.ltrg_GetTuning(0, None) == 0
    finally:
        lib.ltrg_SetTuning(0, C.byref(saved))


@pytest.mark.gpu
def test_results_do_not_depend_on_launch_shape(gpu):
    lib = gpu
    saved = _get(lib)
    d = scenes.mid(5, lm=128, n_boxes=24, n_spheres=3, bounces=0, ao_rays=8)
    try:
        a = bake(lib, d, debug=False)
        t = _get(lib)
        t.direct_block, t.direct_blocks_per_sm, t.ao_block, t.ao_blocks_per_sm = 256, 2, 64, 32
        t.direct_regs = 1 - t.direct_regs   # the other register budget of the shadow-trace kernel
        assert lib.ltrg_SetTuning(0, C.byref(t))
        b = bake(lib, d, debug=False)
        for x, y in zip(a.lightmaps, b.lightmaps):
            np.testing.assert_array_equal(x[3], y[3])
    finally:
        lib.ltrg_SetTuning(0, C.byref(saved))


@pytest.mark.gpu
@pytest.mark.parametrize("shadow_mode", [0, 1])
def test_results_do_not_depend_on_stack_split_or_wavefront(gpu, shadow_mode):
    # the traversal stack's shared-memory part (0, 4, 8, 16 entries), the AO rays per lane
    # per fetch and the warp-cooperative walks change where entries live, which lane traces
    # which ray and which nodes a walk visits, not any query's result
    lib = gpu
    saved = _get(lib)
    d = scenes.mid(5, lm=128, n_boxes=24, n_spheres=3, bounces=0, ao_rays=8)
    opts = {"shadow_mode": shadow_mode}
    try:
        t = _get(lib)
        t.direct_stack, t.ao_stack, t.ao_chunk, t.direct_packet, t.ao_packet = 0, 0, 4, 0, 0
        assert lib.ltrg_SetTuning(0, C.byref(t))
        ref = bake(lib, d, gpu_options=opts)
        for k, chunk, regs, packet in ((4, 1, 0, 0), (8, 2, 1, 1), (16, 8, 0, 1), (0, 4, 2, 1), (0, 1, 3, 0)):
            t.direct_stack, t.ao_stack, t.ao_chunk, t.direct_packet, t.ao_packet = k, k, chunk, packet, packet
            t.direct_regs = t.sampled_regs = regs
            assert lib.ltrg_SetTuning(0, C.byref(t))
            got = bake(lib, d, gpu_options=opts)
            for x, y in zip(ref.lightmaps, got.lightmaps):
                np.testing.assert_array_equal(x[3], y[3])
            for x, y in zip(ref.debug, got.debug):
                np.testing.assert_array_equal(x["vis"], y["vis"])
                np.testing.assert_array_equal(x["ao"], y["ao"])
    finally:
        lib.ltrg_SetTuning(0, C.byref(saved))


@pytest.mark.gpu
@pytest.mark.parametrize("desc", [
    lambda: scenes.mid(5, lm=128, n_boxes=24, n_spheres=3, bounces=1, ao_rays=8),
    lambda: scenes.cornell(3, lm=32, bounces=1, ao=True),
])
def test_results_do_not_depend_on_bvh_builder(gpu, desc):
    # PLOC and the radix hierarchy give different trees over the same leaves in the
    # same order; every query (any hit, closest hit with ties to the lower leaf,
    # nearest distance) and so every texel and AO hit is the same
    d = desc()
    a = bake(gpu, d, gpu_options={"bvh_builder": ext.LTRG_BVH_PLOC, "radiosity_patches": 256, "radiosity_links": 1})
    b = bake(gpu, d, gpu_options={"bvh_builder": ext.LTRG_BVH_RADIX, "radiosity_patches": 256, "radiosity_links": 1})
    for x, y in zip(a.lightmaps, b.lightmaps):
        np.testing.assert_array_equal(x[3], y[3])
    for x, y in zip(a.debug, b.debug):
        np.testing.assert_array_equal(x["pos"], y["pos"])
        if "ao" in x:
            np.testing.assert_array_equal(x["ao"], y["ao"])


@pytest.mark.gpu
def test_trace_orders_change_no_result(gpu):
    # direct_order / ao_order only change which warp traces which pair or ray
    lib = gpu
    saved = _get(lib)
    d = scenes.mid(5, lm=128, n_boxes=24, n_spheres=3, bounces=0, ao_rays=8)
    try:
        res = {}
        for order in (0, 1, 2):
            t = _get(lib)
            t.direct_order = t.ao_order = order
            assert lib.ltrg_SetTuning(0, C.byref(t))
            res[order] = bake(lib, d)
        for order in (1, 2):
            for x, y in zip(res[0].lightmaps, res[order].lightmaps):
                np.testing.assert_array_equal(x[3], y[3])
            for x, y in zip(res[0].debug, res[order].debug):
                np.testing.assert_array_equal(x["vis"], y["vis"])
                np.testing.assert_array_equal(x["ao"], y["ao"])
    finally:
        lib.ltrg_SetTuning(0, C.byref(saved))


@pytest.mark.gpu
def test_autotune_picks_valid_shapes(gpu):
    lib = gpu
    saved = _get(lib)
    h, keep = ingest(lib, scenes.mid(6, lm=128, n_boxes=24, n_spheres=3, bounces=0, ao_rays=8))
    try:
        t = ext.autotune(lib, h)
        assert t["direct_block"] in (64, 128, 256) and t["ao_block"] in (64, 128, 256)
        assert 1 <= t["direct_blocks_per_sm"] <= 64 and 1 <= t["ao_blocks_per_sm"] <= 64
        assert _get(lib).as_dict() == t
        info = ext.Stats()
        assert lib.ltrg_GetStats(h, C.byref(info)) and info.shadow_evals > 0
    finally:
        lib.ltr_DestroyScene(h)
        lib.ltrg_SetTuning(0, C.byref(saved))
