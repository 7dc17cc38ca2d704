"""The bake's radiosity (patch mode, through ltr_Start) against the FP64 Jacobi
oracle, at every form-factor precision.

The GPU bake keeps its radiosity elements (ltrdbg_GetRadiosity: patch
positions, normals, diffuse and area, emitted light, totals and F). The oracle
recomputes every linked factor in double from the same positions and normals
(the links, i.e. the visibility bits, are F's nonzero entries) and iterates
B_k = E + K B_{k-1}, which equals the bake's total = sum_{m<=bounces} K^m E.
Error = max |total - B| / max |B| over all elements and channels.

Bars (the mid scene at 16,691 patches measured 1.4e-7 for FP32 and 1.3e-4
for FP16 with one of two bounces refined):
  FP32 F                         <= 1e-6
  FP16 F, no refinement          <= 1e-3
  BF16 F, no refinement          <= 1e-2
  FP16 / BF16 F, every bounce refined: the FP32 totals bit for bit
FP16 F is stored with a power-of-two scale per row (the Cornell room's
closest patches have factors past FP16's range); the links must survive it.
"""
import ctypes as C
import os

import numpy as np
import pytest

from lighter_gb300 import ext, scenes
from lighter_gb300.scene import ingest

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1


def rad_bake(gpu, desc, **opts):
    scene, keep = ingest(gpu, desc, gpu_options=dict(opts, keep_samples=1))
    try:
        gpu.ltr_Start(scene)
        assert gpu.ltrg_Wait(scene), gpu.ltrg_LastError(scene)
        r = ext.get_radiosity(gpu, scene)
        assert r is not None
        return r
    finally:
        gpu.ltr_DestroyScene(scene)
        del keep


def fp64_total(oracle, r, bounces):
    n = r["n"]
    p = lambda a: np.ascontiguousarray(a, np.float32).ctypes.data_as(C.c_void_p)  # noqa: E731
    out = np.empty((n, 3), np.float64)
    oracle.orc_gather_jacobi_f64.restype = None
    oracle.orc_gather_jacobi_f64(C.c_uint32(n), C.c_uint32(3), p(r["pos"][:, :3]), p(r["nrm"][:, :3]),
                                 p(r["diff_area"][:, 3]), p((r["F"] != 0).astype(np.float32)),
                                 p(r["diff_area"][:, :3]), p(r["emit"][:, :3]), C.c_int(bounces),
                                 out.ctypes.data_as(C.c_void_p), C.c_int(THREADS))
    return out


def err(r, B):
    return float(np.abs(r["total"][:, :3].astype(np.float64) - B).max() / np.abs(B).max())


@pytest.fixture(scope="module")
def room():
    return scenes.cornell(4, lm=32, bounces=3, ao=False)


@pytest.fixture(scope="module")
def room_fp32(gpu, oracle, room):
    r = rad_bake(gpu, room, radiosity_patches=1024, radiosity_links=ext.LTRG_LINKS_VISIBLE)
    return r, fp64_total(oracle, r, 3)


def test_fp32_against_fp64(room_fp32):
    r, B = room_fp32
    assert 512 <= r["n"] <= 2048 and np.count_nonzero(r["F"]) > 0
    print(f"room, {r['n']} patches: FP32 {err(r, B):.3g} against FP64")
    assert err(r, B) <= 1e-6, err(r, B)


@pytest.mark.parametrize("precision,tol", [(ext.LTRG_F_FP16, 1e-3), (ext.LTRG_F_BF16, 1e-2)])
def test_half_precision_against_fp64(gpu, room, room_fp32, precision, tol):
    r32, B = room_fp32
    raw = rad_bake(gpu, room, radiosity_patches=1024, radiosity_links=ext.LTRG_LINKS_VISIBLE,
                   radiosity_precision=precision, refine_steps=0)
    refined = rad_bake(gpu, room, radiosity_patches=1024, radiosity_links=ext.LTRG_LINKS_VISIBLE,
                       radiosity_precision=precision, refine_steps=3)
    assert raw["n"] == r32["n"]
    # same links: the 16-bit F is zero exactly where the FP32 one is
    np.testing.assert_array_equal(raw["F"] != 0, r32["F"] != 0)
    print(f"room: precision {precision} unrefined {err(raw, B):.3g} against FP64")
    assert err(raw, B) <= tol, err(raw, B)
    np.testing.assert_array_equal(refined["total"], r32["total"])


def test_mid_scene_fp16_refined_against_fp64(gpu, oracle):
    # the mid scene at its benchmark size (4 x 1024^2 lightmaps, ~16k patches, 2 bounces)
    d = scenes.mid(seed=1, lm=1024)
    r32 = rad_bake(gpu, d, radiosity_patches=16384, radiosity_links=ext.LTRG_LINKS_VISIBLE)
    B = fp64_total(oracle, r32, 2)
    e32 = err(r32, B)
    r16 = rad_bake(gpu, d, radiosity_patches=16384, radiosity_links=ext.LTRG_LINKS_VISIBLE,
                   radiosity_precision=ext.LTRG_F_FP16, refine_steps=1)
    e16 = err(r16, B)
    print(f"mid scene, {r32['n']} patches: FP32 {e32:.3g}, FP16 + 1 refinement {e16:.3g} against FP64")
    assert e32 <= 1e-6 and e16 <= 1e-3, (e32, e16)
