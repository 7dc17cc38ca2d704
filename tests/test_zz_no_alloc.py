"""ltrg_FinalizeLightmapNoAlloc: the bake's finalize step for callers that
cannot allocate device memory where they finish a lightmap (code inside a
CUDA stream capture, plugins whose host application owns all device memory,
callbacks that must not synchronise the device).

The entry point takes the scattered sample colours and the coverage mask on
the device and writes the finished lightmap, using a fixed scratch array in
the library instead of cudaMalloc. This test feeds it the per-sample colours
of a normal bake (ltr_Start, read back through ltrdbg_GetSamples) and checks
its output against the lightmap that the same bake returned through
ltr_GetWorkOutput, for calls in a row on lightmaps of different sizes (each
call finds the previous one's data in the shared scratch): square ones, a
64 x 32 one (the transposed blur swaps width and height) and a 48 x 80 one
finished without blur (blur_size 0: dilation only).
Collected last (file name) so that a failure here cannot hide other tests.
"""
import ctypes as C

import numpy as np
import pytest

from lighter_gb300 import ext, scenes
from lighter_gb300.scene import bake

pytestmark = pytest.mark.gpu

# same bar as the other lightmap comparisons, tightened: identical kernels
# and inputs, so the outputs must agree to float rounding of one texel
REL_TOL = 1e-6


def _scatter(res, inst):
    d = res.debug[inst]
    uid, _, _, lm, _ = [x for x in res.lightmaps if x[0] == inst][0]
    h, w, _ = lm.shape
    rgb = np.zeros((h * w, 3), np.float32)
    mask = np.zeros(h * w, np.uint8)
    rgb[d["loc"]] = d["color"]
    mask[d["loc"]] = 1
    return rgb, mask, lm, w, h


def test_finalize_no_alloc_matches_bake(gpu):
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available(), "the no-alloc entry point needs a CUDA device"
    # bakes with different lightmap sizes; blur 0.5 is the default config
    res_a = bake(gpu, scenes.cornell(11, lm=64, bounces=0, ao=True))
    res_b = bake(gpu, scenes.cornell(12, lm=32, bounces=0, ao=True))
    d_c = scenes.cornell(13, lm=64, bounces=0, ao=True)
    d_c.fixed_lm_size = (64, 32)
    res_c = bake(gpu, d_c)
    d_d = scenes.cornell(14, lm=64, bounces=0, ao=True)
    d_d.fixed_lm_size = (48, 80)
    d_d.config["blur_size"] = 0.0
    res_d = bake(gpu, d_d)
    stream = torch.cuda.current_stream().cuda_stream
    for res, inst, blur in ((res_a, 1, 0.5), (res_b, 7, 0.5), (res_c, 3, 0.5), (res_d, 2, 0.0)):
        rgb, mask, want, w, h = _scatter(res, inst)
        d_rgb = torch.from_numpy(rgb).cuda()
        d_mask = torch.from_numpy(mask).cuda()
        d_out = torch.full((h * w, 3), float("nan"), dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        rc = gpu.ltrg_FinalizeLightmapNoAlloc(d_rgb.data_ptr(), d_mask.data_ptr(), d_out.data_ptr(), w, h, blur,
                                              C.c_void_p(stream))
        assert rc == ext.NOALLOC_OK
        torch.cuda.synchronize()
        got = d_out.cpu().numpy().reshape(h, w, 3)
        peak = max(float(np.abs(want).max()), 1e-6)
        err = float(np.abs(got - want).max())
        assert err <= REL_TOL * peak, f"instance {inst}: max |no-alloc - bake| = {err:.3g} (peak {peak:.3g})"


def test_finalize_no_alloc_rejects_oversize(gpu):
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    buf = torch.zeros(16, dtype=torch.float32, device="cuda")
    m = torch.zeros(16, dtype=torch.uint8, device="cuda")
    rc = gpu.ltrg_FinalizeLightmapNoAlloc(buf.data_ptr(), m.data_ptr(), buf.data_ptr(), 2048, 1024, 0.5, None)
    assert rc == ext.NOALLOC_ETOOBIG
    rc = gpu.ltrg_FinalizeLightmapNoAlloc(buf.data_ptr(), m.data_ptr(), buf.data_ptr(), 4, 4, 40.0, None)
    assert rc == ext.NOALLOC_EINVAL
