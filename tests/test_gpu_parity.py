"""GPU bake vs the CPU oracle on the same seeded scenes (through the C API).

Tolerances. Stages made only of + - * / sqrt are bit-exact (the library is
built without FMA contraction on host and device). Stages that call
powf/acosf/sinf/cosf/expf differ by CUDA's ulp-level error in those
functions, and a sphere trace or a sample push can amplify an ulp into a
different step count or a different branch at a grazing configuration. The
bars, per lightmap with `peak` = max |oracle|:
  - max |gpu - oracle| over all texels and channels: at most 1e-4 * peak (MAX_TOL);
    a test that allows more names the class of texel that needs it
  - texels with |gpu - oracle| > 1e-3 * peak: at most 1%          (TEXEL_FRAC)
  - mean |gpu - oracle|: at most 2e-4 * peak                      (MEAN_TOL)
  - sample positions bit-identical for at least 99.9% of samples  (POS_FRAC)
Measured (GB300): every texel of the mid scene at 256^2 (the bench's CPU
sample) within 5e-7 of peak, of every other scene here within 5e-6; the
Cornell room at 128^2 is bit-exact.
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
MAX_TOL = 1e-4
POS_FRAC = 0.999


def lightmap_errors(la, lb):
    """(max, mean) |gpu - oracle| of one lightmap relative to the oracle's peak,
    and the fraction of texels (any channel) off by more than TEXEL_RTOL of peak."""
    peak = max(float(np.abs(lb).max()), 1e-6)
    d = np.abs(la - lb)
    frac = float((d.max(-1) > TEXEL_RTOL * peak).mean()) if d.size else 0.0
    return (float(d.max()) / peak if d.size else 0.0), (float(d.mean()) / peak if d.size else 0.0), frac


def compare(rg, ro, name, texel_frac=TEXEL_FRAC, mean_tol=MEAN_TOL, max_tol=MAX_TOL, exact=False):
    assert len(rg.lightmaps) == len(ro.lightmaps), name
    worst = 0.0
    for (ua, ma, ia, la, na), (ub, mb, ib, lb, nb) in zip(rg.lightmaps, ro.lightmaps):
        assert (ua, ma, ia) == (ub, mb, ib)
        assert la.shape == lb.shape, (name, ua)
        if exact:
            np.testing.assert_array_equal(la, lb, err_msg=f"{name} lm {ua}")
            continue
        mx, mean, frac = lightmap_errors(la, lb)
        worst = max(worst, mx)
        assert mx <= max_tol, f"{name} lm {ua}: a texel is off by {mx:.3g} of peak (bar {max_tol:g})"
        assert frac <= texel_frac, f"{name} lm {ua}: {frac:.4f} of texels off by > {TEXEL_RTOL} of peak"
        assert mean <= mean_tol, f"{name} lm {ua}: mean error {mean:.3g} of peak"
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
    print(f"{name}: largest texel error {worst:.3g} of peak")
    return worst


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


def test_bench_cpu_sample_mid256(gpu, oracle):
    """The bench's CPU sample: the full mid scene (400 boxes, 50 icospheres, 10
    lights, AO 32 rays) at 256^2 lightmaps with radiosity off, against the
    oracle on all host threads (its result does not depend on the thread count)."""
    import os
    d = scenes.mid(seed=1, lm=256, bounces=0)
    st = {}
    rg = bake(gpu, d, stats=st)
    ro = bake(oracle, d, threads=os.cpu_count() or 1)
    compare(rg, ro, "mid256", max_tol=1e-5, mean_tol=1e-6, texel_frac=0.0)
    assert st["ao_rays"] == st["samples"] * 32 and st["shadow_evals"] > 100_000


def test_benchmarked_mid1024_direct_and_ao(gpu, oracle):
    """The bench's timed workload at its own size: the mid scene at 4 x 1024^2
    lightmaps with every light and AO 32 rays, radiosity off (the oracle restates
    the reference's per-sample radiosity, which is not runnable at this size; the
    patch radiosity has its own tests), against the oracle on all host threads,
    with the CPU sample's bars."""
    import os
    d = scenes.mid(seed=1, lm=1024, bounces=0)
    st = {}
    rg = bake(gpu, d, stats=st)
    ro = bake(oracle, d, threads=os.cpu_count() or 1)
    compare(rg, ro, "mid1024", max_tol=1e-5, mean_tol=1e-6, texel_frac=0.0)
    assert st["ao_rays"] == st["samples"] * 32 and st["shadow_pairs"] > 1_500_000


def test_c1_cornell_128_bit_exact(gpu, oracle):
    """C1 at its configured 128^2 lightmaps (8 lightmaps, point + directional
    light, no spot light and power 1, so no powf/acosf rounding enters), no
    radiosity: every texel equals the oracle's."""
    import os
    d = scenes.cornell(1, lm=128, bounces=0, ao=False)
    rg = bake(gpu, d)
    ro = bake(oracle, d, threads=os.cpu_count() or 1)
    compare(rg, ro, "c1_128", exact=True)


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


@pytest.mark.parametrize("cfg", [{}, {"ds2x": 1}, {"blur_size": 1.5}])
def test_gpu_rgbe_encoding_matches_the_host_encoder(gpu, cfg):
    """encode_rgbe: the GPU's RGBE images are the host encoder's bytes of the
    float outputs (images.rgbe), with and without downsampling and blur; a bake
    without the option returns none."""
    from lighter_gb300 import images
    d = scenes.cornell(3, lm=64, bounces=1, ao=True)
    d.config.update(cfg)
    res = bake(gpu, d, gpu_options={"encode_rgbe": 1})
    assert len(res.rgbe) == len(res.lightmaps) > 0
    for lm, px in zip(res.lightmaps, res.rgbe):
        np.testing.assert_array_equal(px, images.rgbe(lm[3]))
    assert (np.concatenate([p[..., 3].ravel() for p in res.rgbe]) > 0).any()
    assert bake(gpu, d).rgbe == []


def test_bounce_wait_expiry_fails_the_bake_and_the_next_bake_matches(gpu):
    """The bounce kernel's bounded waits: a bounce whose copy producer issues nothing
    gives up after 20 ms (test limit), the radiosity error word (bit 1) ends that bake
    with an error, and the next bake equals an untouched one bit for bit."""
    d = scenes.cornell(2, lm=32, bounces=2, ao=False)
    opts = {"radiosity_patches": 256, "radiosity_links": 1}
    ref = bake(gpu, d, gpu_options=opts)
    assert gpu.ltrdbg_RadiosityStallNextBounce(20000)
    with pytest.raises(RuntimeError, match="error word 0x00000002"):
        bake(gpu, d, gpu_options=opts)
    again = bake(gpu, d, gpu_options=opts)
    for a, b in zip(ref.lightmaps, again.lightmaps):
        np.testing.assert_array_equal(a[3], b[3])
    assert not gpu.ltrdbg_RadiosityStallNextBounce(0)


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


def test_abort_lands_inside_a_long_trace_launch(gpu):
    """ltr_Abort while one shadow-trace launch runs for more than a second (the
    mid scene at 1024^2 with 8192 sampled shadow rays per pair): the persistent
    warps poll the scene's mapped abort word at every work fetch and stop, so
    the bake ends as "aborted" long before the launch would have finished."""
    import time
    from lighter_gb300.scene import ingest
    d = scenes.mid(2, lm=1024, bounces=0, ao_rays=0)
    for L in d.lights:
        L.shadow_sample_count = 8192
    scene, keep = ingest(gpu, d, gpu_options={"shadow_mode": 1})
    try:
        gpu.ltr_Start(scene)
        assert gpu.ltrg_Wait(scene)
        full = ext.Stats()
        assert gpu.ltrg_GetStats(scene, C.byref(full))
        assert full.ms_direct_trace > 1000.0, full.ms_direct_trace
        # the host queues the whole bake at once (its stage text runs ahead of the GPU),
        # so the abort is timed: well past the sample stage, well inside the trace launch
        ws = abi.WorkStatus()
        gpu.ltr_Start(scene)
        time.sleep(min(0.4, 0.25 * (full.ms_total - full.ms_direct_trace) / 1000.0 + 0.2))
        t0 = time.perf_counter()
        gpu.ltr_Abort(scene)
        assert gpu.ltrg_Wait(scene) == 0
        dt = time.perf_counter() - t0
        assert gpu.ltr_GetStatus(scene, C.byref(ws)) == 0 and ws.stage == b"aborted"
        print(f"abort: bake ended {dt * 1000:.1f} ms after ltr_Abort (full trace launch {full.ms_direct_trace:.0f} ms)")
        assert dt < 0.25 * full.ms_direct_trace / 1000.0
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


@pytest.mark.parametrize("name", ["cornell32", "mid128"])
def test_sampled_soft_shadows(gpu, oracle, name):
    """LTRG_SHADOW_SAMPLED: shadow_sample_count visibility rays per (sample,
    light), restated by the oracle (orc_SetOptions). Both libraries compute the
    light's ray directions and disk points on the host with the same float
    expressions, so each pair's count of occluded rays should agree: fewer than
    0.1% of the rays may flip, and the lightmaps meet the usual bars."""
    import os
    if name == "cornell32":   # point light (16 samples, disk of 0.2 m) + directional light (32 directions)
        d = scenes.cornell(4, lm=32, bounces=0, ao=False)
    else:                     # 8 point + 2 spot lights, 64 samples each
        d = scenes.mid(4, lm=128, n_boxes=24, n_spheres=3, bounces=0, ao_rays=8)
    opts = {"shadow_mode": 1}
    st = {}
    rg = bake(gpu, d, stats=st, gpu_options=opts)
    ro = bake(oracle, d, threads=os.cpu_count() or 1, gpu_options=opts)
    ns = np.array([max(1, L.shadow_sample_count) for L in d.lights], np.int64)[:, None]
    rays = flips = gpu_rays = 0
    for a, b in zip(rg.debug, ro.debug):
        if "vis" not in a or not a["vis"].size:
            continue
        ta, tb = a["vis"] >= 0, b["vis"] >= 0
        assert not (ta & ~tb).any(), f"{name}: pairs traced by the GPU only"
        gpu_rays += int((np.broadcast_to(ns, ta.shape) * ta).sum())
        both = ta & tb
        ha = np.rint((1.0 - a["vis"]) * ns).astype(np.int64)   # occluded rays of the pair
        hb = np.rint((1.0 - b["vis"]) * ns).astype(np.int64)
        rays += int((np.broadcast_to(ns, both.shape) * both).sum())
        flips += int(np.abs(ha - hb)[both].sum())
    assert rays > 0 and st["shadow_evals"] == gpu_rays
    assert flips <= RAY_FLIP_FRAC * rays, f"{name}: {flips} of {rays} shadow rays flip"
    compare(rg, ro, f"sampled_{name}")
    print(f"sampled {name}: {flips}/{rays} shadow rays flip")


def _patch_members(res, n_patches):
    """Patch of every covered sample of a bake, by the patch rule (instance,
    lightmap tile of side t, dominant axis of the unit normal; patches in slot
    order), with t the side whose occupied-slot count equals `n_patches`."""
    insts = res.debug[1:]
    widths = [lm[3].shape[1] for lm in res.lightmaps]
    heights = [lm[3].shape[0] for lm in res.lightmaps]
    axes = []
    for d in insts:
        n = d["nrm"].astype(np.float32)
        l2 = (n[:, 0] * n[:, 0] + n[:, 1] * n[:, 1]) + n[:, 2] * n[:, 2]
        inv = np.float32(1) / np.sqrt(l2, dtype=np.float32)
        nn = n * inv[:, None]
        ax, ay, az = np.abs(nn[:, 0]), np.abs(nn[:, 1]), np.abs(nn[:, 2])
        axes.append(np.where((ax >= ay) & (ax >= az), np.where(nn[:, 0] >= 0, 0, 1),
                             np.where(ay >= az, np.where(nn[:, 1] >= 0, 2, 3), np.where(nn[:, 2] >= 0, 4, 5))))
    for t in range(1, 257):
        base, slots = 0, []
        for d, w, h, ax in zip(insts, widths, heights, axes):
            ntx = (w + t - 1) // t
            loc = d["loc"].astype(np.int64)
            slots.append(base + ((loc // w) // t * ntx + (loc % w) // t) * 6 + ax)
            base += ntx * ((h + t - 1) // t) * 6
        occ = np.unique(np.concatenate(slots))
        if len(occ) == n_patches:
            return [np.searchsorted(occ, sl) for sl in slots]
    raise AssertionError("no tile side gives the patch count")


def test_patch_radiosity_mid256_vs_oracle(gpu, oracle):
    """Patch-mode radiosity (the bench's mode: visible links, patches by
    lightmap tile and normal axis) against the oracle's CPU restatement on the
    full mid scene at 256^2 with 2 bounces. Same patch count (same tile side).
    A patch whose samples all agree with the oracle's (positions and normals
    bit-identical, which the parity bar holds for >= 99.9% of samples) must
    agree to float rounding of its FP64 means; a patch holding one of the few
    samples the sample correction moved differently (box corners) is excluded
    from that bar and counted, and so are the patches it reaches through the
    two bounces' links. Links between agreeing patches: the same set up to
    pairs at the factor or visibility threshold."""
    import os
    d = scenes.mid(seed=1, lm=256, bounces=2)
    opts = {"radiosity_patches": 4096, "radiosity_links": 1}
    st = {}
    rg = bake(gpu, d, stats=st, gpu_options=opts, radiosity=True)
    ro = bake(oracle, d, threads=os.cpu_count() or 1, gpu_options=opts, radiosity=True)
    a, b = rg.radiosity, ro.radiosity
    assert a is not None and b is not None and a["n"] == b["n"] == st["rad_elements"]
    n = a["n"]
    assert 2048 <= n <= 8192
    # patches holding a sample whose GPU position or normal differs from the oracle's
    members = _patch_members(ro, n)
    suspect = np.zeros(n, bool)
    for m, x, y in zip(members, rg.debug[1:], ro.debug[1:]):
        moved = ~((x["pos"] == y["pos"]).all(-1) & (x["nrm"] == y["nrm"]).all(-1))
        suspect[m[moved]] = True
    ok = ~suspect
    assert suspect.sum() <= 0.01 * n, f"{int(suspect.sum())} of {n} patches hold a moved sample"
    for k, rtol in (("pos", 1e-5), ("nrm", 1e-5), ("diff_area", 1e-5), ("emit", 1e-4)):
        np.testing.assert_allclose(a[k][ok], b[k][ok], rtol=rtol, atol=1e-6, err_msg=k)
    la, lb = a["F"] != 0, b["F"] != 0
    both_ok = ok[:, None] & ok[None, :]
    n_links = int(lb[both_ok].sum())
    diff = int((la != lb)[both_ok].sum())
    assert n_links > 0 and diff <= 1e-3 * n_links, f"{diff} of {n_links} links differ"
    both = la & lb & both_ok
    np.testing.assert_allclose(a["F"][both], b["F"][both], rtol=1e-4)
    # a moved patch passes its difference on along its links, one link per bounce
    Fl = lb | la
    reached = suspect.copy()
    for _ in range(2):
        reached |= Fl[:, reached].any(axis=1)
    clean = ~reached
    peak = float(np.abs(b["total"]).max())
    d_tot = np.abs(a["total"] - b["total"]).max(-1) / peak
    print(f"patches {n} ({int(suspect.sum())} hold a moved sample, {int(reached.sum())} within 2 links), "
          f"links {n_links} ({diff} differ), totals: clean {d_tot[clean].max():.3g}, reached "
          f"{d_tot[reached].max() if reached.any() else 0:.3g}, mean {d_tot.mean():.3g} of peak")
    assert d_tot[clean].max() <= 1e-5, "a patch no moved sample reaches differs"
    assert d_tot.max() <= 2e-2 and d_tot.mean() <= 1e-5
    # texels take their patch's bounce: the largest differences sit in reached patches
    compare(rg, ro, "mid256_patches", max_tol=2e-2, mean_tol=1e-5, texel_frac=2e-3)
