"""ctypes mirror of include/lighter_gb300.h (the GPU extensions)."""
import ctypes as C

import numpy as np

from .abi import Config, SampleRequest, u32

LTRG_LINKS_REFERENCE = 0
LTRG_LINKS_VISIBLE = 1
LTRG_F_FP32 = 0
LTRG_F_FP16 = 1
LTRG_F_BF16 = 2
LTRG_BVH_PLOC = 0
LTRG_BVH_RADIX = 1


class Options(C.Structure):
    _fields_ = [
        ("device", C.c_int),
        ("keep_samples", C.c_int),
        ("radiosity_links", C.c_int),
        ("radiosity_precision", C.c_int),
        ("refine_steps", C.c_int),
        ("radiosity_patches", u32),
        ("bvh_builder", u32),
        ("shadow_mode", u32),
        ("intersect_mode", u32),
        ("encode_rgbe", u32),
        ("reserved", u32 * 6),
    ]


class Stats(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "ms_total", "ms_upload", "ms_bvh", "ms_samples", "ms_direct", "ms_rad_links", "ms_rad_bounce", "ms_ao",
        "ms_finalize", "ms_download")] + [(n, C.c_uint64) for n in (
            "texels", "samples", "triangles", "shadow_evals", "distance_queries", "ao_rays", "rad_pairs",
            "rad_vis_rays", "node_visits", "tri_tests", "rad_elements", "kernel_launches", "bytes_h2d",
            "bytes_d2h")] + [("ms_device", C.c_double), ("ms_direct_trace", C.c_double), ("ms_ao_trace", C.c_double),
                             ("shadow_pairs", C.c_uint64), ("reserved", C.c_uint64 * 1)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_ if n != "reserved"}


EXT_API = {
    "ltrg_GetOptions": (None, [C.c_void_p, C.POINTER(Options)]),
    "ltrg_SetOptions": (C.c_int, [C.c_void_p, C.POINTER(Options)]),
    "ltrg_GetStats": (C.c_int, [C.c_void_p, C.POINTER(Stats)]),
    "ltrg_GetWorkOutputRGBE": (C.c_int, [C.c_void_p, u32, C.POINTER(C.POINTER(C.c_ubyte))]),
    "ltrg_LastError": (C.c_char_p, [C.c_void_p]),
    "ltrg_Wait": (C.c_int, [C.c_void_p]),
    "ltrg_StartBatch": (C.c_int, [C.POINTER(C.c_void_p), u32]),
}


class Tuning(C.Structure):
    _fields_ = [("direct_block", u32), ("direct_blocks_per_sm", u32), ("ao_block", u32), ("ao_blocks_per_sm", u32),
                ("direct_order", u32), ("ao_order", u32), ("direct_regs", u32), ("direct_stack", u32),
                ("ao_stack", u32), ("ao_chunk", u32), ("direct_packet", u32), ("sampled_regs", u32),
                ("ao_packet", u32), ("reserved", u32 * 3)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_ if n != "reserved"}


EXT_API.update({
    "ltrg_GetTuning": (C.c_int, [C.c_int, C.POINTER(Tuning)]),
    "ltrg_SetTuning": (C.c_int, [C.c_int, C.POINTER(Tuning)]),
    "ltrg_Autotune": (C.c_int, [C.c_void_p, C.POINTER(Tuning)]),
    "ltrdbg_GetRadiosity": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint32)] + [C.c_void_p] * 6),
    "ltrdbg_TraceSegments": (C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_int, C.c_void_p, C.c_int]),
})

LTRG_ISECT_REFERENCE = 0
LTRG_ISECT_WATERTIGHT = 1
LTRG_SHADOW_SPHERE = 0
LTRG_SHADOW_SAMPLED = 1


def trace_segments(lib, tri_xyz, seg6, intersect_mode=LTRG_ISECT_REFERENCE, device=0):
    """ltrdbg_TraceSegments: closest hit fraction of every segment (n, 6) against
    the triangles (m, 9); 2.0 where a segment hits nothing."""
    tri = np.ascontiguousarray(tri_xyz, dtype=np.float32).reshape(-1, 9)
    seg = np.ascontiguousarray(seg6, dtype=np.float32).reshape(-1, 6)
    out = np.empty(len(seg), np.float32)
    if not lib.ltrdbg_TraceSegments(tri.ctypes.data, len(tri), seg.ctypes.data, len(seg), intersect_mode,
                                    out.ctypes.data, device):
        raise RuntimeError("ltrdbg_TraceSegments failed")
    return out


def get_radiosity(lib, scene, with_F: bool = True):
    """The radiosity elements of the scene's last bake (baked with keep_samples = 1):
    dict of n and (n, 4) float32 arrays pos, nrm, diff_area, emit, total, plus the
    (n, n) form factors F (widened from the stored type) when `with_F`. None when
    the bake ran no radiosity."""
    n = C.c_uint32(0)
    lib.ltrdbg_GetRadiosity(scene, C.byref(n), None, None, None, None, None, None)
    if n.value == 0:
        return None
    out = {k: np.zeros((n.value, 4), np.float32) for k in ("pos", "nrm", "diff_area", "emit", "total")}
    F = np.zeros((n.value, n.value), np.float32) if with_F else None
    ok = lib.ltrdbg_GetRadiosity(scene, C.byref(n), *(out[k].ctypes.data for k in
                                                     ("pos", "nrm", "diff_area", "emit", "total")),
                                 F.ctypes.data if F is not None else None)
    if not ok:
        raise RuntimeError("ltrdbg_GetRadiosity: no radiosity records (F kept only up to 24576 elements)")
    out["n"] = n.value
    out["F"] = F
    return out


def autotune(lib, scene) -> dict:
    """Runs ltrg_Autotune on an ingested scene and returns the chosen launch shapes."""
    t = Tuning()
    if not lib.ltrg_Autotune(scene, C.byref(t)):
        msg = lib.ltrg_LastError(scene)
        raise RuntimeError("autotune failed: " + (msg.decode() if msg else "unknown"))
    return t.as_dict()


def set_options(lib, scene, **kw):
    o = Options()
    lib.ltrg_GetOptions(scene, C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    if not lib.ltrg_SetOptions(scene, C.byref(o)):
        raise ValueError(f"ltrg_SetOptions rejected {kw}")


def get_stats(lib, scene) -> dict:
    s = Stats()
    lib.ltrg_GetStats(scene, C.byref(s))
    return s.as_dict()

# Finalize without device allocation (include/lighter_gb300.h).
NOALLOC_MAX_TEXELS = 1 << 20
NOALLOC_OK, NOALLOC_EINVAL, NOALLOC_ETOOBIG, NOALLOC_ECUDA = 0, -1, -2, -3
EXT_API["ltrg_FinalizeLightmapNoAlloc"] = (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, u32, u32, C.c_float,
                                                     C.c_void_p])

# Multi-right-hand-side radiosity gather (include/lighter_gb300.h).
LTRG_REFINE_NONE = 0
LTRG_REFINE_RHS = 1
LTRG_REFINE_FULL = 2


class GatherStats(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "ms_build", "ms_convert", "ms_bounces", "ms_per_bounce", "ms_gemm", "flops_per_bounce")] + [
        (n, C.c_uint64) for n in ("bytes_per_bounce", "links", "vis_rays", "pairs")] + [
        (n, C.c_int32) for n in ("tensor_cores", "stages", "ctas", "products")] + [("reserved", u32 * 8)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_ if n != "reserved"}


EXT_API.update({
    "ltrg_GatherCreate": (C.c_void_p, [C.c_void_p, u32, C.c_void_p, C.c_void_p, C.c_void_p, u32, C.c_int, C.c_int]),
    "ltrg_GatherDestroy": (None, [C.c_void_p]),
    "ltrg_GatherSetChunk": (C.c_int, [C.c_void_p, u32]),
    "ltrg_GatherSize": (u32, [C.c_void_p]),
    "ltrg_GatherGetG": (C.c_int, [C.c_void_p, C.c_void_p]),
    "ltrg_GatherLastError": (C.c_char_p, [C.c_void_p]),
    "ltrdbg_GatherStallNextSolve": (C.c_int, [C.c_void_p, u32]),
    "ltrdbg_GatherHostPath": (C.c_int, [C.c_void_p, C.c_int]),
    "ltrdbg_GatherHostPathUsed": (C.c_int, [C.c_void_p]),
    "ltrdbg_RadiosityStallNextBounce": (C.c_int, [u32]),
    "ltrdbg_RefTreeDigest": (C.c_int, [C.c_void_p, u32, C.c_int, C.c_void_p]),
    "ltrg_GatherSolve": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, u32, C.c_int, C.c_int, C.c_int, C.c_void_p,
                                   C.POINTER(GatherStats)]),
    "ltrg_GatherSolveDevice": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, u32, C.c_int, C.c_int, C.c_int,
                                         C.c_void_p, C.POINTER(GatherStats), C.c_void_p]),
})
