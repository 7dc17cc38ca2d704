"""Scene description and a driver that bakes it through any ``ltr_*`` library.

`bake(lib, desc)` replays a `SceneDesc` through the public C API exactly as an
application would (lighter_test.cpp:183-544 is the reference's own caller):
create scene, set config, add meshes/parts/instances, seed ``rand()`` and add
lights, add probe samples, ``ltr_Start``, poll ``ltr_GetStatus``, then read the
work outputs. The same driver runs the GPU library, the CPU oracle port and the
reference build, which is what makes their outputs comparable.
"""
from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass, field
from typing import Callable, Optional

import numpy as np

from . import abi

_libc = C.CDLL(None)
_libc.srand.argtypes = [C.c_uint]
_libc.srand.restype = None


def srand(seed: int) -> None:
    """Seed glibc's process-wide rand(); the bake draws one value per light at
    ltr_LightAdd and one per AO texel (lighter.cpp:1300, 819)."""
    _libc.srand(int(seed) & 0xFFFFFFFF)


@dataclass
class Part:
    positions: np.ndarray          # (V,3) f32
    normals: np.ndarray            # (V,3) f32
    uv1: np.ndarray                # (V,2) f32, passed to sample_fn (face id in u)
    uv2: np.ndarray                # (V,2) f32, lightmap UVs
    indices: np.ndarray            # (I,) u32
    shadow: int = 1


@dataclass
class Mesh:
    ident: str
    parts: list


@dataclass
class Instance:
    mesh: int
    matrix: np.ndarray = field(default_factory=lambda: np.eye(4, dtype=np.float32))
    importance: float = 1.0
    shadow: int = 1
    ident: str = ""


@dataclass
class Light:
    type: int
    position: tuple = (0.0, 0.0, 0.0)
    direction: tuple = (0.0, 0.0, 0.0)
    up: tuple = (0.0, 0.0, 0.0)
    color: tuple = (1.0, 1.0, 1.0)
    range: float = 10.0
    power: float = 1.0
    light_radius: float = 0.1
    shadow_sample_count: int = 1
    spot_angle_out: float = 0.0
    spot_angle_in: float = 0.0
    spot_curve: float = 0.0


@dataclass
class SceneDesc:
    name: str
    meshes: list
    instances: list
    lights: list
    config: dict = field(default_factory=dict)
    fixed_lm_size: Optional[tuple] = None          # size_fn forcing (w, h)
    sample_table: Optional[tuple] = None           # (diffuse (F,3), emissive (F,3) or None)
    sample_fn_py: Optional[Callable] = None        # python sample_fn(req) -> bool
    probes: list = field(default_factory=list)     # [(id, pos3, nrm3)]
    seed: int = 1

    def triangle_count(self) -> int:
        n = 0
        for inst in self.instances:
            n += sum(len(p.indices) // 3 for p in self.meshes[inst.mesh].parts)
        return n


@dataclass
class BakeResult:
    lightmaps: list                 # [(uid, mesh_ident, inst_ident, rgb (h,w,3), normals (h,w,4)|None)]
    sample_colors: np.ndarray       # (S,3) probe outputs
    stages: list
    wall_s: float
    debug: list = field(default_factory=list)   # per instance dict of sample arrays
    final_stage: str = ""
    radiosity: Optional[dict] = None             # ext.get_radiosity of the bake (bake(..., radiosity=True))
    rgbe: list = field(default_factory=list)     # per lightmap (h,w,4) uint8 when encode_rgbe was set


def _vec3(v):
    return abi.VEC3(*[float(x) for x in v])


def _has(lib, name):
    try:
        getattr(lib, name)
        return True
    except AttributeError:
        return False


def _populate(lib, scene, desc: SceneDesc, threads: int, keep: list) -> None:
    """Config, meshes, instances, lights (after srand) and probes of `desc`."""
    cfg = abi.Config()
    lib.ltr_GetConfig(C.byref(cfg), scene)
    for k, v in desc.config.items():
        if isinstance(v, (tuple, list)):
            setattr(cfg, k, _vec3(v))
        else:
            setattr(cfg, k, v)
    cfg.max_num_threads = threads
    if desc.fixed_lm_size is not None:
        w, h = desc.fixed_lm_size

        def _size(cfgp, mi, mis, ii, iis, area, imp, out):
            out[0] = w
            out[1] = h
            return 1
        cb = abi.SIZE_FN(_size)
        keep.append(cb)
        cfg.size_fn = C.cast(cb, C.c_void_p).value
    if desc.sample_table is not None:
        dif, emi = desc.sample_table
        dif = np.ascontiguousarray(dif, dtype=np.float32)
        keep.append(dif)
        tab = abi.SampleTable()
        tab.count = dif.shape[0]
        tab.diffuse_rgb = dif.ctypes.data_as(C.POINTER(C.c_float))
        if emi is not None:
            emi = np.ascontiguousarray(emi, dtype=np.float32)
            keep.append(emi)
            tab.emissive_rgb = emi.ctypes.data_as(C.POINTER(C.c_float))
        keep.append(tab)
        cfg.userdata = C.cast(C.pointer(tab), C.c_void_p).value
        cfg.sample_fn = C.cast(lib.ltrg_TableSampleFn, C.c_void_p).value
    elif desc.sample_fn_py is not None:
        fn = desc.sample_fn_py

        def _sample(cfgp, reqp):
            return 1 if fn(reqp.contents) else 0
        cb = abi.SAMPLE_FN(_sample)
        keep.append(cb)
        cfg.sample_fn = C.cast(cb, C.c_void_p).value
    lib.ltr_SetConfig(scene, C.byref(cfg))

    mesh_handles = []
    for m in desc.meshes:
        ident = m.ident.encode()
        mh = lib.ltr_CreateMesh(scene, ident, len(ident))
        mesh_handles.append(mh)
        for p in m.parts:
            pos = np.ascontiguousarray(p.positions, dtype=np.float32)
            nrm = np.ascontiguousarray(p.normals, dtype=np.float32)
            t1 = np.ascontiguousarray(p.uv1, dtype=np.float32)
            t2 = np.ascontiguousarray(p.uv2, dtype=np.float32)
            idx = np.ascontiguousarray(p.indices, dtype=np.uint32)
            info = abi.MeshPartInfo()
            info.positions_f3 = pos.ctypes.data
            info.normals_f3 = nrm.ctypes.data
            info.texcoords1_f2 = t1.ctypes.data
            info.texcoords2_f2 = t2.ctypes.data
            info.stride_positions = 12
            info.stride_normals = 12
            info.stride_texcoords1 = 8
            info.stride_texcoords2 = 8
            info.indices = idx.ctypes.data_as(C.POINTER(abi.u32))
            info.vertex_count = pos.shape[0]
            info.index_count = idx.shape[0]
            info.shadow = int(p.shadow)
            if not lib.ltr_MeshAddPart(mh, C.byref(info)):
                raise RuntimeError(f"ltr_MeshAddPart rejected a part of {m.ident}")
    for inst in desc.instances:
        ii = abi.MeshInstanceInfo()
        mat = np.asarray(inst.matrix, dtype=np.float32).reshape(4, 4)
        for r in range(4):
            for c in range(4):
                ii.matrix[r][c] = float(mat[r, c])
        ii.importance = inst.importance
        ii.shadow = inst.shadow
        ident = inst.ident.encode()
        keep.append(ident)
        ii.ident = ident
        ii.ident_size = len(ident)
        lib.ltr_MeshAddInstance(mesh_handles[inst.mesh], C.byref(ii))

    srand(desc.seed)
    for L in desc.lights:
        li = abi.LightInfo()
        li.type = L.type
        li.position = _vec3(L.position)
        li.direction = _vec3(L.direction)
        li.up_direction = _vec3(L.up)
        li.color_rgb = _vec3(L.color)
        li.range = L.range
        li.power = L.power
        li.light_radius = L.light_radius
        li.shadow_sample_count = L.shadow_sample_count
        li.spot_angle_out = L.spot_angle_out
        li.spot_angle_in = L.spot_angle_in
        li.spot_curve = L.spot_curve
        lib.ltr_LightAdd(scene, C.byref(li))
    for (sid, pos, nrm) in desc.probes:
        si = abi.SampleInfo()
        si.id = sid
        si.position = _vec3(pos)
        si.normal = _vec3(nrm)
        lib.ltr_SampleAdd(scene, C.byref(si))



def ingest(lib, desc: SceneDesc, threads: int = 1, gpu_options: Optional[dict] = None, debug: bool = False):
    """Create a scene and feed `desc` through the C API without starting the
    bake. Returns (scene handle, keep-alive list); the caller keeps the list
    alive while the scene exists (it holds ctypes callbacks and buffers) and
    destroys the scene with ltr_DestroyScene."""
    keep = []
    scene = lib.ltr_CreateScene()
    if not scene:
        raise RuntimeError("ltr_CreateScene returned NULL")
    try:
        _populate(lib, scene, desc, threads, keep)
        if _has(lib, "ltrg_SetOptions"):
            from .ext import set_options
            opts = dict(gpu_options or {})
            if debug:
                opts.setdefault("keep_samples", 1)
            if opts:
                set_options(lib, scene, **opts)
        elif gpu_options and _has(lib, "orc_SetOptions"):
            # the oracle port takes the modes it restates; the other fields
            # (device, tuning, precision) have no meaning on the CPU
            vals = (abi.u32 * len(abi.ORACLE_OPTIONS))(*[int(gpu_options.get(k, 0)) for k in abi.ORACLE_OPTIONS])
            lib.orc_SetOptions(scene, vals, len(abi.ORACLE_OPTIONS))
    except BaseException:
        lib.ltr_DestroyScene(scene)
        raise
    return scene, keep


def bake(lib, desc: SceneDesc, threads: int = 1, debug: bool = True, poll_s: float = 0.001,
         timeout_s: float = 3600.0, before_start: Optional[Callable] = None, gpu_options: Optional[dict] = None,
         stats: Optional[dict] = None, radiosity: bool = False) -> BakeResult:
    """Replay `desc` through `lib`'s C API and return its outputs. For the GPU
    library, `gpu_options` are ltrg_Options fields and `stats` (a dict) receives
    ltrg_GetStats; the oracle port takes the fields of abi.ORACLE_OPTIONS from
    the same dict. A bake that ends in an error raises RuntimeError."""
    scene, keep = ingest(lib, desc, threads, gpu_options, debug)
    try:
        is_gpu = _has(lib, "ltrg_SetOptions")
        if before_start is not None:
            before_start(scene)
        stages = []
        st = abi.WorkStatus()
        t0 = time.perf_counter()
        lib.ltr_Start(scene)
        while lib.ltr_GetStatus(scene, C.byref(st)):
            s = st.stage.decode() if st.stage else ""
            if not stages or stages[-1] != s:
                stages.append(s)
            if time.perf_counter() - t0 > timeout_s:
                lib.ltr_Abort(scene)
            time.sleep(poll_s)
        wall = time.perf_counter() - t0
        final = st.stage.decode() if st.stage else ""
        if is_gpu:
            if final != "finished":
                msg = lib.ltrg_LastError(scene)
                raise RuntimeError(f"bake {desc.name} ended with '{final}': {msg.decode() if msg else ''}")
            if stats is not None:
                from .ext import get_stats
                stats.update(get_stats(lib, scene))

        cfg = abi.Config()
        lib.ltr_GetConfig(C.byref(cfg), scene)
        ao_ns = int(cfg.ao_num_samples) if cfg.ao_distance and cfg.ao_num_samples > 0 else 0
        res = _collect(lib, scene, debug, stages, wall, final, len(desc.lights), ao_ns)
        if radiosity and _has(lib, "ltrdbg_GetRadiosity"):
            # the elements of the radiosity stage; F too while it stays small (n <= 8192)
            from .ext import get_radiosity
            n = abi.u32(0)
            lib.ltrdbg_GetRadiosity(scene, C.byref(n), None, None, None, None, None, None)
            res.radiosity = get_radiosity(lib, scene, with_F=0 < n.value <= 8192)
        return res
    finally:
        lib.ltr_DestroyScene(scene)


def _collect(lib, scene, debug, stages, wall, final, n_lights: int = 0, ao_ns: int = 0) -> "BakeResult":
    info = abi.WorkOutputInfo()
    lib.ltr_GetWorkOutputInfo(scene, C.byref(info))
    lms = []
    for k in range(info.lightmap_count):
        wo = abi.WorkOutput()
        if not lib.ltr_GetWorkOutput(scene, k, C.byref(wo)):
            raise RuntimeError("ltr_GetWorkOutput failed")
        n = wo.width * wo.height
        rgb = np.ctypeslib.as_array(wo.lightmap_rgb, shape=(n * 3,)).copy().reshape(wo.height, wo.width, 3)
        nrm = None
        if wo.normals_xyzf:
            nrm = np.ctypeslib.as_array(wo.normals_xyzf, shape=(n * 4,)).copy().reshape(wo.height, wo.width, 4)
        mid = C.string_at(wo.mesh_ident, wo.mesh_ident_size).decode() if wo.mesh_ident else ""
        iid = C.string_at(wo.inst_ident, wo.inst_ident_size).decode() if wo.inst_ident else ""
        lms.append((wo.uid, mid, iid, rgb, nrm))
    rgbe = []
    if hasattr(lib, "ltrg_GetWorkOutputRGBE"):
        for k, (_, _, _, rgb, _) in enumerate(lms):
            p = C.POINTER(C.c_ubyte)()
            if lib.ltrg_GetWorkOutputRGBE(scene, k, C.byref(p)):
                h, w = rgb.shape[:2]
                rgbe.append(np.ctypeslib.as_array(p, shape=(h * w * 4,)).copy().reshape(h, w, 4))
    colors = np.zeros((info.sample_count, 3), np.float32)
    for k in range(info.sample_count):
        colors[k] = info.samples[k].out_color[:]

    dbg = []
    if debug and hasattr(lib, "ltrdbg_InstanceCount"):
        for i in range(lib.ltrdbg_InstanceCount(scene)):
            n = lib.ltrdbg_SampleCount(scene, i)
            d = {
                "pos": np.zeros((n, 3), np.float32),
                "nrm": np.zeros((n, 3), np.float32),
                "loc": np.zeros((n,), np.uint32),
                "radinfo": np.zeros((n, 4), np.float32),
                "color": np.zeros((n, 3), np.float32),
            }
            if n:
                lib.ltrdbg_GetSamples(scene, i, d["pos"].ctypes.data, d["nrm"].ctypes.data,
                                      d["loc"].ctypes.data, d["radinfo"].ctypes.data, d["color"].ctypes.data)
            if hasattr(lib, "ltrdbg_GetRayData"):
                vis = np.zeros((n_lights, n), np.float32)
                ao = np.zeros((n, ao_ns), np.float32)
                if lib.ltrdbg_GetRayData(scene, i, vis.ctypes.data, ao.ctypes.data if ao_ns else None):
                    d["vis"] = vis
                    if ao_ns:
                        d["ao"] = ao
            dbg.append(d)
    return BakeResult(lms, colors, stages, wall, dbg, final, rgbe=rgbe)


def bake_batch(lib, descs, debug: bool = False, gpu_options: Optional[dict] = None, stats: Optional[list] = None,
               abort: Optional[list] = None):
    """Ingest every scene of `descs` in order, start them as one batch
    (ltrg_StartBatch) and collect their outputs like bake(). Scenes whose
    index is in `abort` get ltr_Abort right after the start; their result is
    None. `stats` (a list) receives one ltrg_GetStats dict per scene."""
    handles = [ingest(lib, d, 1, gpu_options, debug) for d in descs]
    arr = (C.c_void_p * len(handles))(*[h for h, _ in handles])
    try:
        t0 = time.perf_counter()
        if not lib.ltrg_StartBatch(arr, len(handles)):
            raise RuntimeError("ltrg_StartBatch rejected the batch")
        for k in abort or []:
            lib.ltr_Abort(handles[k][0])
        ok = [bool(lib.ltrg_Wait(h)) for h, _ in handles]
        wall = time.perf_counter() - t0
        out = []
        for k, ((h, _), good) in enumerate(zip(handles, ok)):
            st = abi.WorkStatus()
            lib.ltr_GetStatus(h, C.byref(st))
            final = st.stage.decode() if st.stage else ""
            if not good:
                if abort and k in abort:
                    out.append(None)
                    continue
                msg = lib.ltrg_LastError(h)
                raise RuntimeError(f"batch scene {k} ended with '{final}': {msg.decode() if msg else ''}")
            if stats is not None:
                from .ext import get_stats
                stats.append(get_stats(lib, h))
            out.append(_collect(lib, h, debug, [final], wall, final))
        return out, wall
    finally:
        for h, _ in handles:
            lib.ltr_DestroyScene(h)
