"""The C-ABI boundary: exports, struct layouts and host-side behaviour.

No GPU compute runs here: the library is loaded and its host entry points
(configuration, ingest validation, options) are called directly.
"""
import ctypes as C
import os
import re
import subprocess
import tempfile

import pytest

from conftest import REF_SRC, ROOT, has_cuda_device

from lighter_gb300 import abi, ext, scenes
from lighter_gb300.scene import bake

HEADERS = [os.path.join(ROOT, "include", h) for h in ("lighter.h", "lighter_gb300.h")]


def declared_symbols():
    names = set()
    for h in HEADERS:
        txt = open(h).read()
        names |= set(re.findall(r"LTRAPI\s+[\w\s\*]+?\b(ltr\w+)\s*\(", txt))
    return names


def exported_symbols(path):
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True, check=True).stdout
    return {ln.split()[-1] for ln in out.splitlines() if " T " in ln}


def test_library_exports_every_declared_symbol(built):
    from lighter_gb300 import LIB_PATH
    decl = declared_symbols()
    assert set(abi.LTR_API) <= decl   # the 17 entry points of the reference's lighter.h:191-258
    assert len(decl) >= 28
    missing = decl - exported_symbols(LIB_PATH)
    assert not missing, missing


def test_library_loads_and_binds(gpu):
    for name in list(abi.LTR_API) + list(abi.LTRDBG_API) + list(ext.EXT_API):
        assert getattr(gpu, name) is not None


LAYOUT_PROBE = r"""
#include <stdio.h>
#include <stddef.h>
#include "lighter.h"
#define P(T, f) printf(#T "." #f " %zu\n", offsetof(T, f))
#define S(T) printf(#T " %zu\n", sizeof(T))
int main(void) {
  S(ltr_MeshPartInfo); P(ltr_MeshPartInfo, indices); P(ltr_MeshPartInfo, shadow);
  S(ltr_MeshInstanceInfo); P(ltr_MeshInstanceInfo, importance); P(ltr_MeshInstanceInfo, ident_size);
  S(ltr_LightInfo); P(ltr_LightInfo, range); P(ltr_LightInfo, spot_curve);
  S(ltr_SampleInfo); S(ltr_SampleRequest); P(ltr_SampleRequest, part_id); P(ltr_SampleRequest, out_emissive_color);
  S(ltr_Config); P(ltr_Config, max_num_threads); P(ltr_Config, bounce_count); P(ltr_Config, sample_fn);
  P(ltr_Config, ao_num_samples); P(ltr_Config, generate_normalmap_data);
  S(ltr_WorkOutputInfo); S(ltr_WorkOutput); P(ltr_WorkOutput, lightmap_rgb); P(ltr_WorkOutput, height);
  S(ltr_WorkStatus);
  return 0;
}
"""


def _layout(include_dir):
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "probe.cpp")   # the reference header needs C++ (ltr_Config used inside itself)
        exe = os.path.join(d, "probe")
        open(src, "w").write(LAYOUT_PROBE)
        subprocess.run(["g++", "-I", include_dir, src, "-o", exe], check=True, capture_output=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout
    return dict(ln.rsplit(" ", 1) for ln in out.strip().splitlines())


def test_struct_layouts_match_ctypes():
    lay = _layout(os.path.join(ROOT, "include"))
    assert int(lay["ltr_MeshPartInfo"]) == C.sizeof(abi.MeshPartInfo)
    assert int(lay["ltr_MeshInstanceInfo"]) == C.sizeof(abi.MeshInstanceInfo)
    assert int(lay["ltr_LightInfo"]) == C.sizeof(abi.LightInfo)
    assert int(lay["ltr_SampleInfo"]) == C.sizeof(abi.SampleInfo)
    assert int(lay["ltr_SampleRequest"]) == C.sizeof(abi.SampleRequest)
    assert int(lay["ltr_Config"]) == C.sizeof(abi.Config)
    assert int(lay["ltr_WorkOutput"]) == C.sizeof(abi.WorkOutput)
    assert int(lay["ltr_Config.sample_fn"]) == abi.Config.sample_fn.offset
    assert int(lay["ltr_Config.generate_normalmap_data"]) == abi.Config.generate_normalmap_data.offset


def test_struct_layouts_match_reference_header():
    if not os.path.exists(os.path.join(REF_SRC, "lighter.h")):
        pytest.skip("reference header not present")
    assert _layout(os.path.join(ROOT, "include")) == _layout(REF_SRC)


def _cfg(lib, scene=None):
    c = abi.Config()
    lib.ltr_GetConfig(C.byref(c), scene)
    return c


def test_config_defaults_match_oracle(gpu, oracle):
    a, b = _cfg(gpu), _cfg(oracle)
    for name, _ in abi.Config._fields_:
        if name == "size_fn":
            continue
        va, vb = getattr(a, name), getattr(b, name)
        if isinstance(va, C.Array):
            va, vb = list(va), list(vb)
        assert va == vb, name


def test_next_power_of_two_and_default_size(gpu, oracle):
    for x in [1, 2, 3, 5, 64, 65, 1000, 1 << 20, (1 << 20) + 1]:
        assert gpu.ltr_NextPowerOfTwo(x) == oracle.ltr_NextPowerOfTwo(x)
    cfg = _cfg(gpu)
    for area, imp in [(0.0, 1.0), (1.0, 1.0), (100.0, 0.3), (1e6, 1.0), (10.0, 2.0)]:
        o1 = (abi.u32 * 2)()
        o2 = (abi.u32 * 2)()
        r1 = gpu.ltr_DefaultSizeFunc(C.byref(cfg), b"m", 1, b"i", 1, area, imp, o1)
        r2 = oracle.ltr_DefaultSizeFunc(C.byref(cfg), b"m", 1, b"i", 1, area, imp, o2)
        assert r1 == r2 and (not r1 or list(o1) == list(o2))


def _part_info(pos, idx):
    import numpy as np
    pos = np.ascontiguousarray(pos, np.float32)
    idx = np.ascontiguousarray(idx, np.uint32)
    nrm = np.zeros_like(pos)
    uv = np.zeros((len(pos), 2), np.float32)
    info = abi.MeshPartInfo()
    info.positions_f3 = pos.ctypes.data
    info.normals_f3 = nrm.ctypes.data
    info.texcoords1_f2 = uv.ctypes.data
    info.texcoords2_f2 = uv.ctypes.data
    info.stride_positions = info.stride_normals = 12
    info.stride_texcoords1 = info.stride_texcoords2 = 8
    info.indices = idx.ctypes.data_as(C.POINTER(abi.u32))
    info.vertex_count = len(pos)
    info.index_count = len(idx)
    info.shadow = 1
    return info, (pos, idx, nrm, uv)


def test_mesh_add_part_validation(gpu):
    s = gpu.ltr_CreateScene()
    try:
        m = gpu.ltr_CreateMesh(s, b"m", 1)
        ok, keep = _part_info([[0, 0, 0], [1, 0, 0], [0, 1, 0]], [0, 1, 2])
        assert gpu.ltr_MeshAddPart(m, C.byref(ok)) == 1
        two, keep2 = _part_info([[0, 0, 0], [1, 0, 0], [0, 1, 0]], [0, 1])   # reference rule lighter.cpp:1237
        assert gpu.ltr_MeshAddPart(m, C.byref(two)) == 0
        bad, keep3 = _part_info([[0, 0, 0], [1, 0, 0], [0, 1, 0]], [0, 1, 7])   # index past the vertices
        assert gpu.ltr_MeshAddPart(m, C.byref(bad)) == 0
        wo = abi.WorkOutput()
        assert gpu.ltr_GetWorkOutput(s, 0, C.byref(wo)) == 0
    finally:
        gpu.ltr_DestroyScene(s)


def test_options_validation(gpu):
    s = gpu.ltr_CreateScene()
    try:
        o = ext.Options()
        gpu.ltrg_GetOptions(s, C.byref(o))
        assert o.device == 0 and o.radiosity_links == 0 and o.radiosity_precision == 0 and o.refine_steps == 1
        o.radiosity_precision = 7
        assert gpu.ltrg_SetOptions(s, C.byref(o)) == 0
        o.radiosity_precision = 1
        assert gpu.ltrg_SetOptions(s, C.byref(o)) == 1
        assert o.shadow_mode == 0 and o.intersect_mode == 0 and o.encode_rgbe == 0
        for field, bad, good in (("shadow_mode", 2, 1), ("intersect_mode", 2, 1), ("encode_rgbe", 2, 1)):
            setattr(o, field, bad)
            assert gpu.ltrg_SetOptions(s, C.byref(o)) == 0, field
            setattr(o, field, good)
            assert gpu.ltrg_SetOptions(s, C.byref(o)) == 1, field
        back = ext.Options()
        gpu.ltrg_GetOptions(s, C.byref(back))
        assert (back.shadow_mode, back.intersect_mode, back.encode_rgbe) == (1, 1, 1)
        # no bake has run: no encoded outputs
        px = C.POINTER(C.c_ubyte)()
        assert gpu.ltrg_GetWorkOutputRGBE(s, 0, C.byref(px)) == 0
    finally:
        gpu.ltr_DestroyScene(s)


def test_status_before_start(gpu):
    s = gpu.ltr_CreateScene()
    try:
        st = abi.WorkStatus()
        assert gpu.ltr_GetStatus(s, C.byref(st)) == 0
        assert st.stage == b"not started"
    finally:
        gpu.ltr_DestroyScene(s)


def test_bake_without_gpu_fails_loudly(gpu):
    """No CPU fallback: without a CUDA device the bake ends in an error."""
    if has_cuda_device():
        pytest.skip("a CUDA device is present")
    with pytest.raises(RuntimeError, match="no CUDA device"):
        bake(gpu, scenes.basic())


def test_extension_struct_layouts_match_ctypes():
    # every field of the extension structs in include/lighter_gb300.h sits where
    # the ctypes mirror in lighter_gb300/ext.py puts it
    structs = {"ltrg_Options": ext.Options, "ltrg_Stats": ext.Stats, "ltrg_Tuning": ext.Tuning,
               "ltrg_GatherStats": ext.GatherStats}
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "lighter_gb300.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'  printf("{cname} %zu\\n", sizeof({cname}));')
        for f, _ in py._fields_:
            lines.append(f'  printf("{cname}.{f} %zu\\n", offsetof({cname}, {f}));')
    lines += ["  return 0;", "}"]
    with tempfile.TemporaryDirectory() as d:
        src, exe = os.path.join(d, "probe.cpp"), os.path.join(d, "probe")
        open(src, "w").write("\n".join(lines) + "\n")
        subprocess.run(["g++", "-I", os.path.join(ROOT, "include"), src, "-o", exe], check=True, capture_output=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout
    lay = dict(ln.rsplit(" ", 1) for ln in out.strip().splitlines())
    for cname, py in structs.items():
        assert int(lay[cname]) == C.sizeof(py), cname
        for f, _ in py._fields_:
            assert int(lay[f"{cname}.{f}"]) == getattr(py, f).offset, f"{cname}.{f}"
