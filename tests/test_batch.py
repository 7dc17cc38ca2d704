"""Batches of scenes (ltrg_StartBatch): one trace launch per stage for all scenes.

A batch must give every scene exactly the outputs of bakes run one after
another in the batch's order (same kernels per pair and per ray; AO's rand()
draws taken in scene order), so the GPU comparison is bit-exact.
"""
import ctypes as C

import numpy as np
import pytest

from lighter_gb300 import scenes
from lighter_gb300.scene import _collect, bake_batch, ingest


def _sequential(lib, descs):
    handles = [ingest(lib, d) for d in descs]
    try:
        out = []
        for h, _ in handles:
            lib.ltr_Start(h)
            assert lib.ltrg_Wait(h), lib.ltrg_LastError(h)
            out.append(_collect(lib, h, False, [], 0.0, "finished"))
        return out
    finally:
        for h, _ in handles:
            lib.ltr_DestroyScene(h)


def _mixed_batch():
    descs = [scenes.batch_scene(s) for s in (3, 4, 5, 6, 7)]
    descs.insert(2, scenes.cornell(2, lm=32, bounces=0, ao=False))   # no AO: skips the AO rendezvous
    descs.insert(4, scenes.basic())                                   # reference scene: no lights
    return descs


@pytest.mark.gpu
def test_batch_equals_sequential_bakes(gpu):
    descs = _mixed_batch()
    seq = _sequential(gpu, descs)
    stats = []
    bat, wall = bake_batch(gpu, descs, stats=stats)
    assert len(bat) == len(seq)
    for k, (a, b) in enumerate(zip(bat, seq)):
        assert len(a.lightmaps) == len(b.lightmaps)
        for la, lb in zip(a.lightmaps, b.lightmaps):
            np.testing.assert_array_equal(la[3], lb[3], err_msg=f"scene {k} lightmap {la[0]}")
    assert sum(s["ao_rays"] for s in stats) > 0 and sum(s["shadow_evals"] for s in stats) > 0


@pytest.mark.gpu
def test_batch_survives_an_aborted_member(gpu):
    descs = [scenes.batch_scene(s) for s in (11, 12, 13, 14)]
    res, _ = bake_batch(gpu, descs, abort=[1])
    for k, r in enumerate(res):
        if r is not None:
            assert all(np.isfinite(lm[3]).all() for lm in r.lightmaps)
    assert res[0] is not None and res[2] is not None and res[3] is not None


def test_start_batch_rejects_bad_input(built):
    from lighter_gb300 import library
    lib = library()
    h, keep = ingest(lib, scenes.basic())
    try:
        arr = (C.c_void_p * 2)(h, h)
        assert lib.ltrg_StartBatch(arr, 2) == 0          # the same scene twice
        assert lib.ltrg_StartBatch(arr, 0) == 0
        assert lib.ltrg_StartBatch(None, 1) == 0
    finally:
        lib.ltr_DestroyScene(h)


def test_batch_without_gpu_fails_every_scene_without_hanging(built):
    from tests.conftest import has_cuda_device
    if has_cuda_device():
        pytest.skip("checks the no-device path")
    from lighter_gb300 import library
    lib = library()
    handles = [ingest(lib, d) for d in (scenes.basic(), scenes.hugeoverlap(), scenes.basic())]
    try:
        arr = (C.c_void_p * 3)(*[h for h, _ in handles])
        assert lib.ltrg_StartBatch(arr, 3) == 1
        for h, _ in handles:
            assert lib.ltrg_Wait(h) == 0
            assert b"CUDA" in lib.ltrg_LastError(h) or b"device" in lib.ltrg_LastError(h)
    finally:
        for h, _ in handles:
            lib.ltr_DestroyScene(h)
