"""GPU bake vs the CPU oracle on the same seeded scenes (through the C API).

Tolerances. Stages made only of + - * / sqrt are bit-exact (the library is
built without FMA contraction on host and device). Stages that call
powf/acosf/sinf/cosf/expf differ by CUDA's ulp-level error in those
functions, and a sphere trace or a sample push can amplify an ulp into a
different step count or a different branch at a grazing configuration. The
bars, per lightmap with `peak` = max |oracle|:
  - texels with |gpu - oracle| > 1e-3 * peak: at most 1%          (TEXEL_FRAC)
  - mean |gpu - oracle|: at most 2e-4 * peak                      (MEAN_TOL)
  - sample positions bit-identical for at least 99.9% of samples  (POS_FRAC)
"""
import ctypes as C

import numpy as np
import pytest

from lighter_gb300 import abi, ext, scenes
from lighter_gb300.scene import bake

pytestmark = pytest.mark.gpu

TEXEL_RTOL = 1e-3
TEXEL_FRAC = 0.01
MEAN_TOL = 2e-4
POS_FRAC = 0.999


def compare(rg, ro, name, texel_frac=TEXEL_FRAC, mean_tol=MEAN_TOL, exact=False):
    assert len(rg.lightmaps) == len(ro.lightmaps), name
    for (ua, ma, ia, la, na), (ub, mb, ib, lb, nb) in zip(rg.lightmaps, ro.lightmaps):
        assert (ua, ma, ia) == (ub, mb, ib)
        assert la.shape == lb.shape, (name, ua)
        if exact:
            np.testing.assert_array_equal(la, lb, err_msg=f"{name} lm {ua}")
            continue
        peak = max(float(np.abs(lb).max()), 1e-6)
        d = np.abs(la - lb)
        frac = float((d > TEXEL_RTOL * peak).mean())
        assert frac <= texel_frac, f"{name} lm {ua}: {frac:.4f} of texels off by > {TEXEL_RTOL} of peak"
        assert float(d.mean()) <= mean_tol * peak, f"{name} lm {ua}: mean error {d.mean():.3g} (peak {peak:.3g})"
        if na is not None or nb is not None:
            assert na is not None and nb is not None
            dn = np.abs(na - nb)
            assert float((dn > 1e-3).mean()) <= texel_frac, f"{name} normals {ua}"
    # per-sample arrays
    tot = same = 0
    for a, b in zip(rg.debug, ro.debug):
        assert len(a["loc"]) == len(b["loc"]), name
        np.testing.assert_array_equal(a["loc"], b["loc"])
        if len(a["loc"]):
            tot += len(a["loc"])
            same += int((a["pos"] == b["pos"]).all(-1).sum())
    if tot:
        assert same / tot >= POS_FRAC, f"{name}: only {same}/{tot} sample positions identical"
    if len(ro.sample_colors):
        np.testing.assert_allclose(rg.sample_colors, ro.sample_colors, rtol=1e-3, atol=1e-5)


def run_both(gpu, oracle, desc, **opts):
    st = {}
    rg = bake(gpu, desc, stats=st, gpu_options=opts or None)
    ro = bake(oracle, desc)
    return rg, ro, st


@pytest.mark.parametrize("name", ["basic", "hugeoverlap"])
def test_reference_test_scenes_bit_exact(gpu, oracle, name):
    rg, ro, _ = run_both(gpu, oracle, getattr(scenes, name)())
    compare(rg, ro, name, exact=True)
    for a, b in zip(rg.debug, ro.debug):
        for k in a:
            np.testing.assert_array_equal(a[k], b[k], err_msg=f"{name}:{k}")


def test_cornell_direct_and_ao(gpu, oracle):
    rg, ro, st = run_both(gpu, oracle, scenes.cornell(3, lm=32, bounces=0, ao=True))
    compare(rg, ro, "cornell32_ao")
    assert st["shadow_evals"] > 0 and st["ao_rays"] == st["samples"] * 17


def test_cornell_radiosity_reference_links(gpu, oracle):
    d = scenes.cornell(3, lm=32, bounces=1, ao=False)
    d.probes = [(7, (5.0, 5.0, 1.0), (0.0, 0.0, 1.0)), (9, (2.0, 8.0, 3.0), (1.0, 0.0, 0.0))]
    rg, ro, st = run_both(gpu, oracle, d)
    compare(rg, ro, "cornell32_rad", texel_frac=0.02)
    assert st["rad_elements"] == st["samples"]


def test_spot_lights_and_many_instances(gpu, oracle):
    rg, ro, _ = run_both(gpu, oracle, scenes.mid(3, lm=128, n_boxes=16, n_spheres=2, bounces=0, ao_rays=8))
    compare(rg, ro, "mid128")


def test_large_terrain_scaled_down(gpu, oracle):
    # the C3 generator (fBm terrain tiles + rocks packed into each tile's lightmap) at a small size;
    # the oracle's result does not depend on its thread count
    import os
    d = scenes.large(2, lm=64, grid=(64, 32), n_rocks=40, n_points=4, ao_rays=4, bounces=0)
    st = {}
    rg = bake(gpu, d, stats=st)
    ro = bake(oracle, d, threads=os.cpu_count() or 1)
    compare(rg, ro, "large64")
    assert st["triangles"] == d.triangle_count() and len(rg.lightmaps) == 16


def test_normal_map_and_blur(gpu, oracle):
    d = scenes.cornell(5, lm=32, bounces=0, ao=True)
    d.config.update(generate_normalmap_data=1, blur_size=1.5)
    rg, ro, _ = run_both(gpu, oracle, d)
    compare(rg, ro, "cornell_normals_blur")
    assert all(x[4] is not None for x in rg.lightmaps)


def test_downsample(gpu, oracle):
    d = scenes.cornell(6, lm=32, bounces=0, ao=False)
    d.config.update(ds2x=1)
    rg, ro, _ = run_both(gpu, oracle, d)
    compare(rg, ro, "cornell_ds2x")
    assert rg.lightmaps[0][3].shape == (16, 16, 3)


def test_ao_effect_negative_and_falloff(gpu, oracle):
    d = scenes.cornell(8, lm=32, bounces=0, ao=True)
    d.config.update(ao_effect=-0.5, ao_falloff=2.0, ao_color_rgb=(0.2, 0.1, 0.05), ao_num_samples=40,
                    ambient_color=(0.05, 0.05, 0.05))
    rg, ro, _ = run_both(gpu, oracle, d)
    compare(rg, ro, "cornell_ao_effect")


def test_repeat_bake_is_deterministic(gpu):
    d = scenes.cornell(9, lm=32, bounces=1, ao=True)
    a = bake(gpu, d)
    b = bake(gpu, d)
    for x, y in zip(a.lightmaps, b.lightmaps):
        np.testing.assert_array_equal(x[3], y[3])


def test_patch_radiosity_runs_and_adds_light(gpu):
    d = scenes.cornell(2, lm=32, bounces=2, ao=False)
    st = {}
    with_rad = bake(gpu, d, stats=st, gpu_options={"radiosity_patches": 256, "radiosity_links": 1})
    d0 = scenes.cornell(2, lm=32, bounces=0, ao=False)
    no_rad = bake(gpu, d0)
    assert 128 <= st["rad_elements"] <= 512   # the tile side is picked for the count closest to 256
    gain = sum(float(x[3].sum()) for x in with_rad.lightmaps) - sum(float(x[3].sum()) for x in no_rad.lightmaps)
    assert gain > 0


@pytest.mark.parametrize("precision,tol", [(1, 1e-3), (2, 4e-3)])
def test_half_precision_form_factors_and_refinement(gpu, precision, tol):
    # 16-bit F: with refine_steps = bounces every bounce recomputes its factors in FP32 (F is
    # only the link mask), which is the FP32 bake bit for bit; without refinement the
    # lightmaps stay within `tol` of the peak (FP16 rounds a factor by <= 2^-11, BF16 2^-8)
    d = scenes.cornell(3, lm=32, bounces=2, ao=False)
    f32 = bake(gpu, d, gpu_options={"radiosity_precision": 0})
    refined = bake(gpu, d, gpu_options={"radiosity_precision": precision, "refine_steps": 2})
    raw = bake(gpu, d, gpu_options={"radiosity_precision": precision, "refine_steps": 0})
    for a, b, c in zip(f32.lightmaps, refined.lightmaps, raw.lightmaps):
        np.testing.assert_array_equal(a[3], b[3])
        peak = float(np.abs(a[3]).max())
        assert float(np.abs(c[3] - a[3]).max()) <= tol * peak


def test_invalid_option_rejected_and_error_reported(gpu):
    s = gpu.ltr_CreateScene()
    try:
        o = ext.Options()
        gpu.ltrg_GetOptions(s, C.byref(o))
        o.device = 99
        assert gpu.ltrg_SetOptions(s, C.byref(o)) == 1      # validated at ltr_Start
        gpu.ltr_Start(s)
        assert gpu.ltrg_Wait(s) == 0
        st = abi.WorkStatus()
        assert gpu.ltr_GetStatus(s, C.byref(st)) == 0
        assert st.stage.startswith(b"error")
        assert b"device" in gpu.ltrg_LastError(s)
    finally:
        gpu.ltr_DestroyScene(s)


def test_abort_between_stages(gpu):
    """ltr_Abort (a no-op in the reference, lighter.cpp:1154-1157) ends the
    bake at the next stage boundary with stage "aborted" and no outputs; the
    scene can be baked again afterwards."""
    from lighter_gb300.scene import ingest
    d = scenes.cornell(3, lm=128, bounces=1, ao=True)   # seconds of work: the abort lands mid-bake
    scene, keep = ingest(gpu, d)
    try:
        gpu.ltr_Start(scene)
        gpu.ltr_Abort(scene)
        assert gpu.ltrg_Wait(scene) == 0
        st = abi.WorkStatus()
        assert gpu.ltr_GetStatus(scene, C.byref(st)) == 0
        assert st.stage == b"aborted"
        info = abi.WorkOutputInfo()
        gpu.ltr_GetWorkOutputInfo(scene, C.byref(info))
        assert info.lightmap_count == 0
        gpu.ltr_Start(scene)   # a later bake of the same scene runs to completion
        assert gpu.ltrg_Wait(scene) == 1
        gpu.ltr_GetWorkOutputInfo(scene, C.byref(info))
        assert info.lightmap_count == 8
    finally:
        gpu.ltr_DestroyScene(scene)
        del keep


RAY_FLIP_FRAC = 1e-3   # fewer than 0.1% of shadow / AO rays may flip hit/miss (grazing-edge cases only)


def _ray_flips(rg, ro):
    """(AO rays, AO flips, traced shadow pairs, blocked/unblocked flips, pairs traced by the GPU only).
    The GPU skips pairs whose unshadowed term is zero (a directional light facing away), which
    the reference and the oracle trace and then multiply by zero; those are not mismatches."""
    ao_tot = ao_flip = sh_tot = sh_flip = traced_mismatch = 0
    for a, b in zip(rg.debug, ro.debug):
        if "ao" in a and "ao" in b and a["ao"].size:
            ha, hb = a["ao"] < 1.0, b["ao"] < 1.0
            ao_tot += ha.size
            ao_flip += int((ha != hb).sum())
        if "vis" in a and "vis" in b and a["vis"].size:
            ta, tb = a["vis"] >= 0, b["vis"] >= 0
            traced_mismatch += int((ta & ~tb).sum())
            both = ta & tb
            sh_tot += int(both.sum())
            sh_flip += int(((a["vis"] == 0) != (b["vis"] == 0))[both].sum())
    return ao_tot, ao_flip, sh_tot, sh_flip, traced_mismatch


@pytest.mark.parametrize("name", ["cornell32_ao", "mid128", "large64"])
def test_shadow_and_ao_rays_flip_below_a_thousandth(gpu, oracle, name):
    import os
    if name == "cornell32_ao":
        d = scenes.cornell(4, lm=32, bounces=0, ao=True)
    elif name == "mid128":
        d = scenes.mid(4, lm=128, n_boxes=24, n_spheres=3, bounces=0, ao_rays=8)
    else:
        d = scenes.large(3, lm=64, grid=(64, 32), n_rocks=40, n_points=4, ao_rays=4, bounces=0)
    rg = bake(gpu, d)
    ro = bake(oracle, d, threads=os.cpu_count() or 1)
    ao_tot, ao_flip, sh_tot, sh_flip, mism = _ray_flips(rg, ro)
    assert ao_tot > 0 and sh_tot > 0
    assert ao_flip <= RAY_FLIP_FRAC * ao_tot, f"{name}: {ao_flip} of {ao_tot} AO rays flip"
    assert sh_flip <= RAY_FLIP_FRAC * sh_tot, f"{name}: {sh_flip} of {sh_tot} shadow pairs flip"
    assert mism <= RAY_FLIP_FRAC * sh_tot, f"{name}: {mism} pairs traced by the GPU only"
    print(f"{name}: AO {ao_flip}/{ao_tot} flips, shadow {sh_flip}/{sh_tot} flips, traced-set mismatch {mism}")
