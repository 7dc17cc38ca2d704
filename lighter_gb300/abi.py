"""ctypes mirror of the lighter C ABI (include/lighter.h).

The struct layouts follow archo5/lighter's lighter.h:64-233 field for field, so
the same Python code drives any library that exports the ``ltr_*`` API: the
GPU baker (liblighter_gb300.so), the CPU oracle port and the reference build.
"""
import ctypes as C

u32 = C.c_uint32
VEC3 = C.c_float * 3
MAT4 = (C.c_float * 4) * 4

LTR_LT_POINT = 1
LTR_LT_SPOT = 2
LTR_LT_DIRECT = 3


class MeshPartInfo(C.Structure):
    _fields_ = [
        ("positions_f3", C.c_void_p),
        ("normals_f3", C.c_void_p),
        ("texcoords1_f2", C.c_void_p),
        ("texcoords2_f2", C.c_void_p),
        ("stride_positions", u32),
        ("stride_normals", u32),
        ("stride_texcoords1", u32),
        ("stride_texcoords2", u32),
        ("indices", C.POINTER(u32)),
        ("vertex_count", u32),
        ("index_count", u32),
        ("shadow", C.c_int),
    ]


class MeshInstanceInfo(C.Structure):
    _fields_ = [
        ("matrix", MAT4),
        ("importance", C.c_float),
        ("shadow", C.c_int),
        ("ident", C.c_char_p),
        ("ident_size", C.c_size_t),
    ]


class LightInfo(C.Structure):
    _fields_ = [
        ("type", u32),
        ("position", VEC3),
        ("direction", VEC3),
        ("up_direction", VEC3),
        ("color_rgb", VEC3),
        ("range", C.c_float),
        ("power", C.c_float),
        ("light_radius", C.c_float),
        ("shadow_sample_count", C.c_int),
        ("spot_angle_out", C.c_float),
        ("spot_angle_in", C.c_float),
        ("spot_curve", C.c_float),
    ]


class SampleInfo(C.Structure):
    _fields_ = [
        ("id", u32),
        ("position", VEC3),
        ("normal", VEC3),
        ("out_color", VEC3),
    ]


class SampleRequest(C.Structure):
    _fields_ = [
        ("position", VEC3),
        ("normal", VEC3),
        ("tex0u", C.c_float), ("tex0v", C.c_float),
        ("tex1u", C.c_float), ("tex1v", C.c_float),
        ("part_id", u32),
        ("mesh_ident", C.c_char_p),
        ("mesh_ident_size", C.c_size_t),
        ("inst_ident", C.c_char_p),
        ("inst_ident_size", C.c_size_t),
        ("out_diffuse_color", VEC3),
        ("out_emissive_color", VEC3),
    ]


class Config(C.Structure):
    pass


SIZE_FN = C.CFUNCTYPE(C.c_int, C.POINTER(Config), C.c_char_p, C.c_size_t, C.c_char_p, C.c_size_t,
                      C.c_float, C.c_float, C.POINTER(u32))
SAMPLE_FN = C.CFUNCTYPE(C.c_int, C.POINTER(Config), C.POINTER(SampleRequest))

Config._fields_ = [
    ("userdata", C.c_void_p),
    ("size_fn", C.c_void_p),
    ("max_num_threads", C.c_int),
    ("max_tree_memory", C.c_size_t),
    ("max_lightmap_size", u32),
    ("default_width", u32),
    ("default_height", u32),
    ("global_size_factor", C.c_float),
    ("max_correct_dist", C.c_float),
    ("max_correct_angle", C.c_float),
    ("clear_color", VEC3),
    ("ambient_color", VEC3),
    ("bounce_count", C.c_int),
    ("sample_fn", C.c_void_p),
    ("ao_distance", C.c_float),
    ("ao_multiplier", C.c_float),
    ("ao_falloff", C.c_float),
    ("ao_effect", C.c_float),
    ("ao_divergence", C.c_float),
    ("ao_color_rgb", VEC3),
    ("ao_num_samples", C.c_int),
    ("blur_size", C.c_float),
    ("ds2x", C.c_int),
    ("generate_normalmap_data", C.c_int),
]


class WorkOutputInfo(C.Structure):
    _fields_ = [
        ("lightmap_count", u32),
        ("sample_count", u32),
        ("samples", C.POINTER(SampleInfo)),
    ]


class WorkOutput(C.Structure):
    _fields_ = [
        ("uid", u32),
        ("mesh_ident", C.c_void_p),
        ("mesh_ident_size", C.c_size_t),
        ("inst_ident", C.c_void_p),
        ("inst_ident_size", C.c_size_t),
        ("lightmap_rgb", C.POINTER(C.c_float)),
        ("normals_xyzf", C.POINTER(C.c_float)),
        ("width", u32),
        ("height", u32),
    ]


class WorkStatus(C.Structure):
    _fields_ = [("completion", C.c_float), ("stage", C.c_char_p)]


class SampleTable(C.Structure):
    """userdata layout read by ``ltrg_TableSampleFn``: per-face albedo/emission
    selected by the integer part of the request's first UV channel."""
    _fields_ = [
        ("count", u32),
        ("diffuse_rgb", C.POINTER(C.c_float)),
        ("emissive_rgb", C.POINTER(C.c_float)),
    ]


# Every entry point of include/lighter.h: name -> (restype, argtypes).
LTR_API = {
    "ltr_CreateScene": (C.c_void_p, []),
    "ltr_DestroyScene": (None, [C.c_void_p]),
    "ltr_Start": (None, [C.c_void_p]),
    "ltr_Abort": (None, [C.c_void_p]),
    "ltr_GetStatus": (C.c_int, [C.c_void_p, C.POINTER(WorkStatus)]),
    "ltr_Sleep": (None, [C.c_int]),
    "ltr_GetConfig": (None, [C.POINTER(Config), C.c_void_p]),
    "ltr_SetConfig": (C.c_int, [C.c_void_p, C.POINTER(Config)]),
    "ltr_CreateMesh": (C.c_void_p, [C.c_void_p, C.c_char_p, C.c_size_t]),
    "ltr_MeshAddPart": (C.c_int, [C.c_void_p, C.POINTER(MeshPartInfo)]),
    "ltr_MeshAddInstance": (C.c_int, [C.c_void_p, C.POINTER(MeshInstanceInfo)]),
    "ltr_LightAdd": (None, [C.c_void_p, C.POINTER(LightInfo)]),
    "ltr_SampleAdd": (None, [C.c_void_p, C.POINTER(SampleInfo)]),
    "ltr_GetWorkOutputInfo": (None, [C.c_void_p, C.POINTER(WorkOutputInfo)]),
    "ltr_GetWorkOutput": (C.c_int, [C.c_void_p, u32, C.POINTER(WorkOutput)]),
    "ltr_NextPowerOfTwo": (u32, [u32]),
    "ltr_DefaultSizeFunc": (C.c_int, [C.POINTER(Config), C.c_char_p, C.c_size_t, C.c_char_p, C.c_size_t,
                                      C.c_float, C.c_float, C.POINTER(u32)]),
}

# Read-only per-stage introspection shared by the GPU library and both CPU checkers.
LTRDBG_API = {
    "ltrdbg_InstanceCount": (u32, [C.c_void_p]),
    "ltrdbg_SampleCount": (u32, [C.c_void_p, u32]),
    "ltrdbg_LightmapSize": (C.c_int, [C.c_void_p, u32, C.POINTER(u32)]),
    "ltrdbg_GetSamples": (C.c_int, [C.c_void_p, u32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "ltrdbg_RadLinkCount": (u32, [C.c_void_p]),
    "ltrg_TableSampleFn": (C.c_int, [C.POINTER(Config), C.POINTER(SampleRequest)]),
}


# Bound where the library has them (the GPU library and the oracle port; not the reference build).
LTRDBG_OPTIONAL = {
    "ltrdbg_GetRayData": (C.c_int, [C.c_void_p, u32, C.c_void_p, C.c_void_p]),
    # the oracle port's switch for the modes beyond the reference (shadow_mode,
    # intersect_mode, radiosity_patches, radiosity_links)
    "orc_SetOptions": (None, [C.c_void_p, C.POINTER(u32), u32]),
    "ltrdbg_GetRadiosity": (C.c_int, [C.c_void_p, C.POINTER(u32)] + [C.c_void_p] * 6),
}

# ltrg_Options fields the oracle port also understands, in orc_SetOptions order.
ORACLE_OPTIONS = ("shadow_mode", "intersect_mode", "radiosity_patches", "radiosity_links")


def bind(lib, table):
    for name, (res, args) in table.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib
